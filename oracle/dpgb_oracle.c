/* Test infrastructure only: the CPU oracle (see dpgb_oracle.h).  Used by the
 * tests, the smoke check and the CPU-baseline leg of bench.py as the checker;
 * never linked into the product.  Plain C11 + OpenMP, FP64 unless a function
 * says otherwise.  Citations are paths in the deepmodeling/deepmd-kit tree. */
#include "dpgb_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* tabulate_fusion_se_a: table interval location, quintic evaluation and the
 * sorted-padding fold, restated from source/lib/src/tabulate.cc:45-160
 * (locate_xx, polynomial5, polynomial5_grad) and 162-449 (the three
 * se_a kernels with NDESCRPT = 4).  Instantiated for double and float with
 * the same operation order as the reference so that the FP32 form matches. */
#define ORC_TAB_DEFINE(T, SFX, NEXTAFTER)                                       \
  static void locate_##SFX(T lower, T upper, T mx, T s0, T s1, T* xx, int* idx, \
                           T* delta) {                                         \
    const T orig = *xx;                                                        \
    *delta = (T)0.;                                                            \
    if (*xx < lower) {                                                         \
      *idx = 0;                                                                \
      *xx = (T)0.;                                                             \
      *delta = orig - lower;                                                   \
    } else if (*xx < upper) {                                                  \
      *idx = (int)((*xx - lower) / s0);                                        \
      *xx -= (*idx * s0 + lower);                                              \
    } else if (*xx < mx) {                                                     \
      int first = (int)((upper - lower) / s0);                                 \
      *idx = first + (int)((*xx - upper) / s1);                                \
      *xx -= ((*idx - first) * s1 + upper);                                    \
    } else {                                                                   \
      int first = (int)((upper - lower) / s0);                                 \
      const T bxx = NEXTAFTER(mx, lower);                                      \
      *idx = first + (int)((bxx - upper) / s1);                                \
      *xx = mx - ((*idx - first) * s1 + upper);                                \
      *delta = orig - mx;                                                      \
    }                                                                          \
  }                                                                            \
  static inline T poly5_##SFX(const T* a, T x) {                               \
    return a[0] + (a[1] + (a[2] + (a[3] + (a[4] + a[5] * x) * x) * x) * x) * x; \
  }                                                                            \
  static inline T poly5g_##SFX(const T* a, T x) {                              \
    return a[1] + ((T)2. * a[2] +                                              \
                   ((T)3. * a[3] + ((T)4. * a[4] + (T)5. * a[5] * x) * x) *   \
                       x) *                                                    \
                      x;                                                       \
  }                                                                            \
  void orc_tabulate_fusion_se_a_##SFX(T* out, const T* table, const T* info,   \
                                      const T* em_x, const T* em, int nloc,    \
                                      int nnei, int nl, int is_sorted) {       \
    memset(out, 0, sizeof(T) * (size_t)nloc * 4 * nl);                         \
    if (nnei <= 0) return;                                                     \
    const T lower = info[0], upper = info[1], mx = info[2], s0 = info[3],      \
            s1 = info[4];                                                      \
    _Pragma("omp parallel for") for (int ii = 0; ii < nloc; ++ii) {            \
      const T ago = em_x[(size_t)ii * nnei + nnei - 1];                        \
      int unloop = 0;                                                          \
      for (int jj = 0; jj < nnei; ++jj) {                                      \
        const T* ll = em + ((size_t)ii * nnei + jj) * 4;                       \
        T xx = em_x[(size_t)ii * nnei + jj];                                   \
        if (ago == xx && ll[1] == 0. && ll[2] == 0. && ll[3] == 0. &&         \
            is_sorted)                                                         \
          unloop = 1;                                                          \
        int idx = 0;                                                           \
        T delta = (T)0.;                                                       \
        locate_##SFX(lower, upper, mx, s0, s1, &xx, &idx, &delta);             \
        for (int kk = 0; kk < nl; ++kk) {                                      \
          const T* a = table + (size_t)idx * nl * 6 + 6 * kk;                  \
          const T g = poly5g_##SFX(a, xx);                                     \
          const T var = poly5_##SFX(a, xx) + g * delta;                        \
          const T scale = unloop ? (nnei - jj) * var : var;                    \
          for (int mm = 0; mm < 4; ++mm)                                       \
            out[(size_t)ii * nl * 4 + mm * nl + kk] += scale * ll[mm];         \
        }                                                                      \
        if (unloop) break;                                                     \
      }                                                                        \
    }                                                                          \
  }                                                                            \
  void orc_tabulate_fusion_se_a_grad_##SFX(                                    \
      T* dy_dem_x, T* dy_dem, const T* table, const T* info, const T* em_x,    \
      const T* em, const T* dy, int nloc, int nnei, int nl, int is_sorted) {   \
    if (nnei <= 0) return;                                                     \
    memset(dy_dem_x, 0, sizeof(T) * (size_t)nloc * nnei);                      \
    memset(dy_dem, 0, sizeof(T) * (size_t)nloc * nnei * 4);                    \
    const T lower = info[0], upper = info[1], mx = info[2], s0 = info[3],      \
            s1 = info[4];                                                      \
    _Pragma("omp parallel for") for (int ii = 0; ii < nloc; ++ii) {            \
      const T ago = em_x[(size_t)ii * nnei + nnei - 1];                        \
      int unloop = 0;                                                          \
      for (int jj = 0; jj < nnei; ++jj) {                                      \
        const size_t eb = ((size_t)ii * nnei + jj) * 4;                        \
        const T* ll = em + eb;                                                 \
        T xx = em_x[(size_t)ii * nnei + jj];                                   \
        if (ago == xx && ll[1] == 0. && ll[2] == 0. && ll[3] == 0. &&         \
            is_sorted)                                                         \
          unloop = 1;                                                          \
        int idx = 0;                                                           \
        T delta = (T)0.;                                                       \
        locate_##SFX(lower, upper, mx, s0, s1, &xx, &idx, &delta);             \
        T grad = (T)0.;                                                        \
        for (int kk = 0; kk < nl; ++kk) {                                      \
          T rr[4];                                                             \
          for (int mm = 0; mm < 4; ++mm)                                       \
            rr[mm] = dy[(size_t)ii * nl * 4 + mm * nl + kk];                   \
          const T* a = table + (size_t)idx * nl * 6 + 6 * kk;                  \
          const T g = poly5g_##SFX(a, xx);                                     \
          const T res = poly5_##SFX(a, xx) + g * delta;                        \
          T dot = (T)0.;                                                       \
          for (int mm = 0; mm < 4; ++mm) dot += ll[mm] * rr[mm];               \
          if (unloop) {                                                        \
            grad += g * dot * (nnei - jj);                                     \
            for (int mm = 0; mm < 4; ++mm)                                     \
              dy_dem[eb + mm] += res * rr[mm] * (nnei - jj);                   \
          } else {                                                             \
            grad += g * dot;                                                   \
            for (int mm = 0; mm < 4; ++mm) dy_dem[eb + mm] += res * rr[mm];    \
          }                                                                    \
        }                                                                      \
        dy_dem_x[(size_t)ii * nnei + jj] = grad;                               \
        if (unloop) break;                                                     \
      }                                                                        \
    }                                                                          \
  }                                                                            \
  void orc_tabulate_fusion_se_a_grad_grad_##SFX(                               \
      T* dz_dy, const T* table, const T* info, const T* em_x, const T* em,     \
      const T* dz_dy_dem_x, const T* dz_dy_dem, int nloc, int nnei, int nl,    \
      int is_sorted) {                                                         \
    memset(dz_dy, 0, sizeof(T) * (size_t)nloc * 4 * nl);                       \
    if (nnei <= 0) return;                                                     \
    const T lower = info[0], upper = info[1], mx = info[2], s0 = info[3],      \
            s1 = info[4];                                                      \
    _Pragma("omp parallel for") for (int ii = 0; ii < nloc; ++ii) {            \
      const T ago = em_x[(size_t)ii * nnei + nnei - 1];                        \
      int unloop = 0;                                                          \
      for (int jj = 0; jj < nnei; ++jj) {                                      \
        const size_t eb = ((size_t)ii * nnei + jj) * 4;                        \
        const T* ll = em + eb;                                                 \
        const T* hh = dz_dy_dem + eb;                                          \
        T xx = em_x[(size_t)ii * nnei + jj];                                   \
        const T dz_xx = dz_dy_dem_x[(size_t)ii * nnei + jj];                   \
        if (ago == xx && ll[1] == 0. && ll[2] == 0. && ll[3] == 0. &&         \
            is_sorted)                                                         \
          unloop = 1;                                                          \
        int idx = 0;                                                           \
        T delta = (T)0.;                                                       \
        locate_##SFX(lower, upper, mx, s0, s1, &xx, &idx, &delta);             \
        for (int kk = 0; kk < nl; ++kk) {                                      \
          const T* a = table + (size_t)idx * nl * 6 + 6 * kk;                  \
          const T vg = poly5g_##SFX(a, xx);                                    \
          const T var = poly5_##SFX(a, xx) + vg * delta;                       \
          const T scale = unloop ? (T)(nnei - jj) : (T)1.;                     \
          for (int mm = 0; mm < 4; ++mm)                                       \
            dz_dy[(size_t)ii * nl * 4 + mm * nl + kk] +=                       \
                scale * (var * hh[mm] + (dz_xx * vg + (T)0.) * ll[mm]);        \
        }                                                                      \
        if (unloop) break;                                                     \
      }                                                                        \
    }                                                                          \
  }

ORC_TAB_DEFINE(double, f64, nextafter)
ORC_TAB_DEFINE(float, f32, nextafterf)

/* ------------------------------------------------------------------------ */
/* Switching function s(r) = u^3(-6u^2+15u-10)+1 on [rmin, rmax] and its
 * derivative: source/lib/include/switcher.h spline5_switch and
 * deepmd/pt/utils/preprocess.py:9-19 compute_smooth_weight. */
static void spline5(double xx, double rmin, double rmax, double* vv,
                    double* dd) {
  if (xx < rmin) {
    *dd = 0.;
    *vv = 1.;
  } else if (xx < rmax) {
    const double uu = (xx - rmin) / (rmax - rmin);
    const double du = 1. / (rmax - rmin);
    *vv = uu * uu * uu * (-6. * uu * uu + 15. * uu - 10.) + 1.;
    *dd = (3. * uu * uu * (-6. * uu * uu + 15. * uu - 10.) +
           uu * uu * uu * (-12. * uu + 15.)) *
          du;
  } else {
    *dd = 0.;
    *vv = 0.;
  }
}

/* The C++ library's switch takes the radii as float references, so the
 * interval width rmax - rmin is a float subtraction
 * (source/lib/include/switcher.h spline5_switch, env_mat.cc:132-133). */
static void spline5_fr(double xx, float rmin, float rmax, double* vv, double* dd) {
  if (xx < rmin) {
    *dd = 0.;
    *vv = 1.;
  } else if (xx < rmax) {
    const float w = rmax - rmin;
    const double uu = (xx - rmin) / w;
    const double du = 1. / w;
    *vv = uu * uu * uu * (-6. * uu * uu + 15. * uu - 10.) + 1.;
    *dd = (3. * uu * uu * (-6. * uu * uu + 15. * uu - 10.) +
           uu * uu * uu * (-12. * uu + 15.)) *
          du;
  } else {
    *dd = 0.;
    *vv = 0.;
  }
}

/* The 4-vector R~ = s(r)[1/r, x/r^2, y/r^2, z/r^2] of a displacement d =
 * r_j - r_i and its derivative with respect to the CENTRE atom (the sign
 * convention of source/lib/src/env_mat.cc:156-216), deriv[c*3+k]. */
static void env_row_sw(const double d[3], double rmin, double rmax, int float_radii,
                       double em[4], double deriv[12]) {
  const double nr2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  const double inr = 1. / sqrt(nr2);
  const double nr = nr2 * inr;
  const double inr2 = inr * inr;
  const double inr4 = inr2 * inr2;
  const double inr3 = inr4 * nr;
  double sw, dsw;
  if (float_radii)
    spline5_fr(nr, (float)rmin, (float)rmax, &sw, &dsw);
  else
    spline5(nr, rmin, rmax, &sw, &dsw);
  const double v0 = 1. / nr;
  const double v[3] = {d[0] / nr2, d[1] / nr2, d[2] / nr2};
  for (int k = 0; k < 3; ++k)
    deriv[k] = d[k] * inr3 * sw - v0 * dsw * d[k] * inr;
  for (int c = 0; c < 3; ++c)
    for (int k = 0; k < 3; ++k)
      deriv[3 + c * 3 + k] =
          (2. * d[c] * d[k] * inr4 - (c == k ? inr2 : 0.)) * sw -
          v[c] * dsw * d[k] * inr;
  em[0] = v0 * sw;
  for (int c = 0; c < 3; ++c) em[1 + c] = v[c] * sw;
}

static void env_row(const double d[3], double rmin, double rmax, double em[4],
                    double deriv[12]) {
  env_row_sw(d, rmin, rmax, 0, em, deriv);
}

/* source/lib/src/env_mat.cc:123-223 with the normalisation of
 * prod_env_mat.cc:102-118.  The reference stops each type section at its
 * first -1; formatted lists keep -1 trailing per section, so evaluating every
 * non-negative slot is the same. */
void orc_env_mat_a(double* em, double* em_deriv, double* rij,
                   const double* coord_ext, const int* atype_ext,
                   const int* nlist, const double* davg, const double* dstd,
                   int nloc, int nnei, double rcut, double rcut_smth) {
#pragma omp parallel for
  for (int ii = 0; ii < nloc; ++ii) {
    const int ti = atype_ext[ii];
    for (int jj = 0; jj < nnei; ++jj) {
      const size_t s = (size_t)ii * nnei + jj;
      const int jx = nlist[s];
      double e4[4] = {0, 0, 0, 0}, dv[12], d[3] = {0, 0, 0};
      memset(dv, 0, sizeof(dv));
      if (jx >= 0) {
        for (int k = 0; k < 3; ++k)
          d[k] = coord_ext[(size_t)jx * 3 + k] - coord_ext[(size_t)ii * 3 + k];
        env_row_sw(d, rcut_smth, rcut, 1, e4, dv);
      }
      for (int k = 0; k < 3; ++k) rij[s * 3 + k] = d[k];
      for (int c = 0; c < 4; ++c) {
        const double a = ti >= 0 ? davg[((size_t)ti * nnei + jj) * 4 + c] : 0.;
        const double sd = ti >= 0 ? dstd[((size_t)ti * nnei + jj) * 4 + c] : 1.;
        em[s * 4 + c] = ti >= 0 ? (e4[c] - a) / sd : 0.;
        for (int k = 0; k < 3; ++k)
          em_deriv[s * 12 + c * 3 + k] = ti >= 0 ? dv[c * 3 + k] / sd : 0.;
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* Neighbour ordering. */
typedef struct {
  int type;
  double key;
  int index;
} nbr_t;

static int cmp_type_key_index(const void* pa, const void* pb) {
  const nbr_t* a = (const nbr_t*)pa;
  const nbr_t* b = (const nbr_t*)pb;
  if (a->type != b->type) return a->type < b->type ? -1 : 1;
  if (a->key != b->key) return a->key < b->key ? -1 : 1;
  if (a->index != b->index) return a->index < b->index ? -1 : 1;
  return 0;
}

static int cmp_key_index(const void* pa, const void* pb) {
  const nbr_t* a = (const nbr_t*)pa;
  const nbr_t* b = (const nbr_t*)pb;
  if (a->key != b->key) return a->key < b->key ? -1 : 1;
  if (a->index != b->index) return a->index < b->index ? -1 : 1;
  return 0;
}

/* source/lib/src/fmt_nlist.cc:98-150 (format_nlist_i_cpu): FP32 squared
 * distance, (type, r2, index) order, rcut2 inclusive, per-type truncation. */
int orc_format_nlist_cpp(int* nlist, const double* coord, const int* atype,
                         const int* in_rows, const int* in_counts, int max_nbor,
                         int nloc, int nall, double rcut, const int* sel,
                         int ntypes) {
  int nnei = 0, sec[ORC_MAX_TYPES + 1];
  sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) sec[t + 1] = sec[t] + sel[t];
  nnei = sec[ntypes];
  int overflow = 0;
  (void)nall;
#pragma omp parallel for reduction(+ : overflow)
  for (int ii = 0; ii < nloc; ++ii) {
    nbr_t* buf = (nbr_t*)malloc(sizeof(nbr_t) * (size_t)(max_nbor > 0 ? max_nbor : 1));
    int n = 0;
    const float rc = (float)rcut;
    const float rcut2 = rc * rc;
    for (int kk = 0; kk < in_counts[ii]; ++kk) {
      const int j = in_rows[(size_t)ii * max_nbor + kk];
      if (atype[j] < 0) continue;
      float df[3];
      for (int d = 0; d < 3; ++d)
        df[d] = (float)coord[(size_t)j * 3 + d] - (float)coord[(size_t)ii * 3 + d];
      const float r2 = df[0] * df[0] + df[1] * df[1] + df[2] * df[2];
      if (r2 <= rcut2) {
        buf[n].type = atype[j];
        buf[n].key = (double)r2;
        buf[n].index = j;
        ++n;
      }
    }
    qsort(buf, (size_t)n, sizeof(nbr_t), cmp_type_key_index);
    int iter[ORC_MAX_TYPES];
    for (int t = 0; t < ntypes; ++t) iter[t] = sec[t];
    for (int jj = 0; jj < nnei; ++jj) nlist[(size_t)ii * nnei + jj] = -1;
    int ov = 0;
    for (int kk = 0; kk < n; ++kk) {
      const int t = buf[kk].type;
      if (iter[t] < sec[t + 1])
        nlist[(size_t)ii * nnei + iter[t]++] = buf[kk].index;
      else
        ov = 1;
    }
    overflow += ov;
    free(buf);
  }
  return overflow;
}

/* deepmd/pt/utils/nlist.py:49-199 (build_neighbor_list with
 * distinguish_types) + 304-337 (nlist_distinguish_types), as a binned search
 * over the extended atoms instead of the dense distance matrix.  Ties in
 * distance are broken by the extended index. */
int orc_build_nlist_pt(int* nlist, const double* coord_ext, const int* atype_ext,
                       int nloc, int nall, double rcut, const int* sel,
                       int ntypes) {
  int sec[ORC_MAX_TYPES + 1];
  sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) sec[t + 1] = sec[t] + sel[t];
  const int nnei = sec[ntypes];
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int a = 0; a < nall; ++a) {
    if (atype_ext[a] < 0) continue;
    for (int d = 0; d < 3; ++d) {
      const double x = coord_ext[(size_t)a * 3 + d];
      if (x < lo[d]) lo[d] = x;
      if (x > hi[d]) hi[d] = x;
    }
  }
  int nb[3];
  for (int d = 0; d < 3; ++d) {
    if (hi[d] < lo[d]) { lo[d] = 0; hi[d] = 0; }
    nb[d] = (int)((hi[d] - lo[d]) / rcut) + 1;
    if (nb[d] > 256) nb[d] = 256;
  }
  const size_t ncell = (size_t)nb[0] * nb[1] * nb[2];
  int* head = (int*)malloc(sizeof(int) * (ncell + 1));
  int* cell_of = (int*)malloc(sizeof(int) * (size_t)(nall > 0 ? nall : 1));
  int* order = (int*)malloc(sizeof(int) * (size_t)(nall > 0 ? nall : 1));
  double csz[3];
  for (int d = 0; d < 3; ++d) csz[d] = (hi[d] - lo[d]) / nb[d] + 1e-12;
  memset(head, 0, sizeof(int) * (ncell + 1));
  for (int a = 0; a < nall; ++a) {
    if (atype_ext[a] < 0) { cell_of[a] = -1; continue; }
    int c[3];
    for (int d = 0; d < 3; ++d) {
      c[d] = (int)((coord_ext[(size_t)a * 3 + d] - lo[d]) / csz[d]);
      if (c[d] < 0) c[d] = 0;
      if (c[d] >= nb[d]) c[d] = nb[d] - 1;
    }
    cell_of[a] = (c[0] * nb[1] + c[1]) * nb[2] + c[2];
    head[cell_of[a] + 1]++;
  }
  for (size_t c = 0; c < ncell; ++c) head[c + 1] += head[c];
  {
    int* fill = (int*)malloc(sizeof(int) * (ncell + 1));
    memcpy(fill, head, sizeof(int) * (ncell + 1));
    for (int a = 0; a < nall; ++a)
      if (cell_of[a] >= 0) order[fill[cell_of[a]]++] = a;
    free(fill);
  }
  /* cells reach: a cell is csz wide, a neighbour may be rcut away */
  int reach[3];
  for (int d = 0; d < 3; ++d) reach[d] = (int)ceil(rcut / csz[d]);
#pragma omp parallel
  {
    size_t cap = 1024;
    nbr_t* buf = (nbr_t*)malloc(sizeof(nbr_t) * cap);
#pragma omp for schedule(dynamic, 16)
    for (int ii = 0; ii < nloc; ++ii) {
      for (int jj = 0; jj < nnei; ++jj) nlist[(size_t)ii * nnei + jj] = -1;
      if (atype_ext[ii] < 0) continue;
      const double* ri = coord_ext + (size_t)ii * 3;
      const int ci = cell_of[ii];
      const int cx = ci / (nb[1] * nb[2]), cy = (ci / nb[2]) % nb[1],
                cz = ci % nb[2];
      size_t n = 0;
      for (int x = cx - reach[0]; x <= cx + reach[0]; ++x) {
        if (x < 0 || x >= nb[0]) continue;
        for (int y = cy - reach[1]; y <= cy + reach[1]; ++y) {
          if (y < 0 || y >= nb[1]) continue;
          for (int z = cz - reach[2]; z <= cz + reach[2]; ++z) {
            if (z < 0 || z >= nb[2]) continue;
            const int c = (x * nb[1] + y) * nb[2] + z;
            for (int p = head[c]; p < head[c + 1]; ++p) {
              const int a = order[p];
              if (a == ii) continue;
              const double dx = coord_ext[(size_t)a * 3 + 0] - ri[0];
              const double dy = coord_ext[(size_t)a * 3 + 1] - ri[1];
              const double dz = coord_ext[(size_t)a * 3 + 2] - ri[2];
              /* the FMA chain of torch.linalg.norm on the CPU, so that
               * near-equal distances order as in the reference */
              const double r = sqrt(fma(dz, dz, fma(dy, dy, dx * dx)));
              if (r <= rcut) {
                if (n == cap) {
                  cap *= 2;
                  buf = (nbr_t*)realloc(buf, sizeof(nbr_t) * cap);
                }
                buf[n].type = atype_ext[a];
                buf[n].key = r;
                buf[n].index = a;
                ++n;
              }
            }
          }
        }
      }
      qsort(buf, n, sizeof(nbr_t), cmp_key_index);
      if (n > (size_t)nnei) n = (size_t)nnei; /* topk(sum(sel)) */
      int iter[ORC_MAX_TYPES];
      for (int t = 0; t < ntypes; ++t) iter[t] = sec[t];
      for (size_t k = 0; k < n; ++k) {
        const int t = buf[k].type;
        if (t >= 0 && t < ntypes && iter[t] < sec[t + 1])
          nlist[(size_t)ii * nnei + iter[t]++] = buf[k].index;
      }
    }
    free(buf);
  }
  free(head);
  free(cell_of);
  free(order);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* source/lib/src/prod_force.cc:23-87 */
void orc_prod_force_a(double* force, const double* net_deriv,
                      const double* env_deriv, const int* nlist, int nloc,
                      int nall, int nnei) {
  const int nd = 4 * nnei;
  memset(force, 0, sizeof(double) * (size_t)nall * 3);
  for (int i = 0; i < nloc; ++i) {
    for (int a = 0; a < nd; ++a)
      for (int k = 0; k < 3; ++k)
        force[(size_t)i * 3 + k] -=
            net_deriv[(size_t)i * nd + a] * env_deriv[((size_t)i * nd + a) * 3 + k];
    for (int j = 0; j < nnei; ++j) {
      const int jx = nlist[(size_t)i * nnei + j];
      if (jx < 0) continue;
      for (int a = 4 * j; a < 4 * j + 4; ++a)
        for (int k = 0; k < 3; ++k)
          force[(size_t)jx * 3 + k] +=
              net_deriv[(size_t)i * nd + a] *
              env_deriv[((size_t)i * nd + a) * 3 + k];
    }
  }
}

/* source/lib/src/prod_virial.cc:22-69 */
void orc_prod_virial_a(double* virial, double* atom_virial,
                       const double* net_deriv, const double* env_deriv,
                       const double* rij, const int* nlist, int nloc, int nall,
                       int nnei) {
  const int nd = 4 * nnei;
  memset(virial, 0, sizeof(double) * 9);
  memset(atom_virial, 0, sizeof(double) * (size_t)nall * 9);
  for (int i = 0; i < nloc; ++i)
    for (int j = 0; j < nnei; ++j) {
      const int jx = nlist[(size_t)i * nnei + j];
      if (jx < 0) continue;
      for (int a = 4 * j; a < 4 * j + 4; ++a) {
        const double pref = -net_deriv[(size_t)i * nd + a];
        for (int d0 = 0; d0 < 3; ++d0)
          for (int d1 = 0; d1 < 3; ++d1) {
            const double v = pref * rij[((size_t)i * nnei + j) * 3 + d1] *
                             env_deriv[((size_t)i * nd + a) * 3 + d0];
            virial[d0 * 3 + d1] -= v;
            atom_virial[(size_t)jx * 9 + d0 * 3 + d1] -= v;
          }
      }
    }
}

/* source/lib/src/prod_force_grad.cc: d(force)/d(net_deriv) contracted with a
 * force cotangent `grad` [nloc(+ghost) , 3] read at local and neighbour rows. */
void orc_prod_force_grad_a(double* grad_net, const double* grad,
                           const double* env_deriv, const int* nlist, int nloc,
                           int nnei) {
  const int nd = 4 * nnei;
  memset(grad_net, 0, sizeof(double) * (size_t)nloc * nd);
  for (int i = 0; i < nloc; ++i) {
    for (int a = 0; a < nd; ++a)
      for (int k = 0; k < 3; ++k)
        grad_net[(size_t)i * nd + a] -=
            grad[(size_t)i * 3 + k] * env_deriv[((size_t)i * nd + a) * 3 + k];
    for (int j = 0; j < nnei; ++j) {
      int jx = nlist[(size_t)i * nnei + j];
      if (jx >= nloc) jx = jx % nloc;
      if (jx < 0) continue;
      for (int a = 4 * j; a < 4 * j + 4; ++a)
        for (int k = 0; k < 3; ++k)
          grad_net[(size_t)i * nd + a] +=
              grad[(size_t)jx * 3 + k] * env_deriv[((size_t)i * nd + a) * 3 + k];
    }
  }
}

/* source/lib/src/prod_virial_grad.cc */
void orc_prod_virial_grad_a(double* grad_net, const double* grad,
                            const double* env_deriv, const double* rij,
                            const int* nlist, int nloc, int nnei) {
  const int nd = 4 * nnei;
  memset(grad_net, 0, sizeof(double) * (size_t)nloc * nd);
  for (int i = 0; i < nloc; ++i)
    for (int j = 0; j < nnei; ++j) {
      const int jx = nlist[(size_t)i * nnei + j];
      if (jx < 0) continue;
      for (int a = 4 * j; a < 4 * j + 4; ++a)
        for (int d0 = 0; d0 < 3; ++d0)
          for (int d1 = 0; d1 < 3; ++d1)
            grad_net[(size_t)i * nd + a] -=
                -1.0 * grad[d0 * 3 + d1] * rij[((size_t)i * nnei + j) * 3 + d1] *
                env_deriv[((size_t)i * nd + a) * 3 + d0];
    }
}

/* ------------------------------------------------------------------------ */
/* MLP layers (deepmd/pt/model/network/mlp.py:188-219): y = tanh(xW+b)[*idt]
 * (+ x when widths match, + [x,x] when the output doubles). */
static void layer_fwd(const double* W, const double* b, const double* idt,
                      int nin, int nout, const double* x, double* t,
                      double* y) {
  for (int o = 0; o < nout; ++o) {
    double pre = b ? b[o] : 0.;
    for (int i = 0; i < nin; ++i) pre += x[i] * W[(size_t)i * nout + o];
    t[o] = tanh(pre);
    y[o] = idt ? t[o] * idt[o] : t[o];
    if (nout == nin)
      y[o] += x[o];
    else if (nout == 2 * nin)
      y[o] += x[o % nin];
  }
}

static void layer_bwd(const double* W, const double* idt, int nin, int nout,
                      const double* t, const double* dy, double* dx,
                      double* scratch) {
  for (int o = 0; o < nout; ++o)
    scratch[o] = dy[o] * (idt ? idt[o] : 1.) * (1. - t[o] * t[o]);
  for (int i = 0; i < nin; ++i) {
    double s = 0.;
    for (int o = 0; o < nout; ++o) s += W[(size_t)i * nout + o] * scratch[o];
    if (nout == nin)
      s += dy[i];
    else if (nout == 2 * nin)
      s += dy[i] + dy[i + nin];
    dx[i] = s;
  }
}

#define ORC_MAXW 2048

/* Embedding net of one neighbour: G(x) and, optionally, x-gradient. */
static void emb_eval(const orc_se_a_model* m, int net, double x, double* G,
                     double* acts /* [n_emb][ORC_MAXW] tanh values */) {
  double buf[2][ORC_MAXW];
  double* cur = buf[0];
  cur[0] = x;
  int nin = 1;
  for (int l = 0; l < m->n_emb; ++l) {
    const int nout = m->emb_neuron[l];
    double* nxt = (l == m->n_emb - 1) ? G : buf[(l + 1) & 1];
    layer_fwd(m->emb_w[net][l], m->emb_b[net][l], m->emb_idt[net][l], nin,
              nout, cur, acts + (size_t)l * ORC_MAXW, nxt);
    if (l < m->n_emb - 1) {
      cur = nxt;
    }
    nin = nout;
  }
}

static double emb_backprop(const orc_se_a_model* m, int net, const double* acts,
                           const double* dG) {
  double bufa[ORC_MAXW], bufb[ORC_MAXW], scratch[ORC_MAXW];
  const double* dy = dG;
  double* dx = bufa;
  for (int l = m->n_emb - 1; l >= 0; --l) {
    const int nout = m->emb_neuron[l];
    const int nin = l == 0 ? 1 : m->emb_neuron[l - 1];
    layer_bwd(m->emb_w[net][l], m->emb_idt[net][l], nin, nout,
              acts + (size_t)l * ORC_MAXW, dy, dx, scratch);
    dy = dx;
    dx = (dx == bufa) ? bufb : bufa;
  }
  return dy[0];
}

/* Fitting net of one atom: returns e and, when dD != NULL, de/dD. */
static double fit_eval(const orc_se_a_model* m, int t, const double* D,
                       double* dD, double* acts /* [n_fit][ORC_MAXW] */,
                       double* hs /* [n_fit+1][ORC_MAXW] inputs per layer */) {
  const int nd = m->dim_descrpt;
  memcpy(hs, D, sizeof(double) * nd);
  int nin = nd;
  for (int l = 0; l < m->n_fit; ++l) {
    const int nout = m->fit_neuron[l];
    layer_fwd(m->fit_w[t][l], m->fit_b[t][l], m->fit_idt[t][l], nin, nout,
              hs + (size_t)l * ORC_MAXW, acts + (size_t)l * ORC_MAXW,
              hs + (size_t)(l + 1) * ORC_MAXW);
    nin = nout;
  }
  const double* wl = m->fit_w[t][m->n_fit];
  const double* hl = hs + (size_t)m->n_fit * ORC_MAXW;
  double e = m->fit_b[t][m->n_fit] ? m->fit_b[t][m->n_fit][0] : 0.;
  for (int i = 0; i < nin; ++i) e += hl[i] * wl[i];
  if (dD && m->n_fit == 0) {
    for (int i = 0; i < nin; ++i) dD[i] = wl[i];
  } else if (dD) {
    double bufa[ORC_MAXW], bufb[ORC_MAXW], scratch[ORC_MAXW];
    for (int i = 0; i < nin; ++i) bufa[i] = wl[i];
    double* dy = bufa;
    double* dx = bufb;
    for (int l = m->n_fit - 1; l >= 0; --l) {
      const int nout = m->fit_neuron[l];
      const int li = l == 0 ? nd : m->fit_neuron[l - 1];
      double* tgt = (l == 0) ? dD : dx;
      layer_bwd(m->fit_w[t][l], m->fit_idt[t][l], li, nout,
                acts + (size_t)l * ORC_MAXW, dy, tgt, scratch);
      if (l > 0) {
        double* tmp = dy;
        dy = dx;
        dx = tmp;
      }
    }
  }
  return e;
}

int orc_se_a_energy_force(const orc_se_a_model* m, const double* coord_ext,
                          const int* atype_ext, const int* nlist, int nloc,
                          int nall, double* atom_energy, double* force_ext,
                          double* virial, double* atom_virial_ext,
                          double* descriptor, double* rot_mat) {
  const int nt = m->ntypes;
  int sec[ORC_MAX_TYPES + 1];
  sec[0] = 0;
  for (int t = 0; t < nt; ++t) sec[t + 1] = sec[t] + m->sel[t];
  const int nnei = sec[nt];
  const int ng = m->emb_neuron[m->n_emb - 1];
  const int M = m->axis_neuron;
  const int nd = m->dim_descrpt;
  if (ng > ORC_MAXW || nd > ORC_MAXW) return 1;
  double* gpair = (double*)calloc((size_t)nloc * nnei * 3, sizeof(double));
  double* dpair = (double*)calloc((size_t)nloc * nnei * 3, sizeof(double));
  if (!gpair || !dpair) return 2;

#pragma omp parallel
  {
    double* Rn = (double*)malloc(sizeof(double) * (size_t)nnei * 4);
    double* dRn = (double*)malloc(sizeof(double) * (size_t)nnei * 4);
    double* der = (double*)malloc(sizeof(double) * (size_t)nnei * 12);
    double* xyz = (double*)malloc(sizeof(double) * 4 * ng);
    double* dxyz = (double*)malloc(sizeof(double) * 4 * ng);
    double* D = (double*)malloc(sizeof(double) * nd);
    double* dD = (double*)malloc(sizeof(double) * nd);
    double* G = (double*)malloc(sizeof(double) * ORC_MAXW);
    double* dG = (double*)malloc(sizeof(double) * ORC_MAXW);
    double* eacts = (double*)malloc(sizeof(double) * ORC_MAX_LAYERS * ORC_MAXW);
    double* facts = (double*)malloc(sizeof(double) * (ORC_MAX_LAYERS + 1) * ORC_MAXW);
    double* fhs = (double*)malloc(sizeof(double) * (ORC_MAX_LAYERS + 2) * ORC_MAXW);
    /* compressed-form scratch: one section at a time */
    double* sec_out = (double*)malloc(sizeof(double) * 4 * ng);
    double* sec_dx = (double*)malloc(sizeof(double) * (size_t)nnei);
    double* sec_dem = (double*)malloc(sizeof(double) * (size_t)nnei * 4);
    double* sec_x = (double*)malloc(sizeof(double) * (size_t)nnei);
#pragma omp for schedule(dynamic, 4)
    for (int i = 0; i < nloc; ++i) {
      const int ti = atype_ext[i];
      if (ti < 0) {
        atom_energy[i] = 0.;
        if (descriptor) memset(descriptor + (size_t)i * nd, 0, sizeof(double) * nd);
        if (rot_mat) memset(rot_mat + (size_t)i * ng * 3, 0, sizeof(double) * ng * 3);
        continue;
      }
      /* env matrix, PyTorch semantics (env_mat.py:18-55,115-118): every
       * non-negative slot is evaluated; padding gives (0-avg)/std */
      for (int j = 0; j < nnei; ++j) {
        const size_t s = (size_t)i * nnei + j;
        const int e = nlist[s];
        double e4[4] = {0, 0, 0, 0}, dv[12];
        memset(dv, 0, sizeof(dv));
        if (e >= 0) {
          double d[3];
          for (int k = 0; k < 3; ++k)
            d[k] = coord_ext[(size_t)e * 3 + k] - coord_ext[(size_t)i * 3 + k];
          env_row(d, m->rcut_smth, m->rcut, e4, dv);
          for (int k = 0; k < 3; ++k) dpair[s * 3 + k] = d[k];
        }
        int keep = 1;
        if (m->pair_mask && e >= 0) keep = m->pair_mask[ti * nt + atype_ext[e]];
        for (int c = 0; c < 4; ++c) {
          const double a = m->davg[((size_t)ti * nnei + j) * 4 + c];
          const double sd = m->dstd[((size_t)ti * nnei + j) * 4 + c];
          Rn[j * 4 + c] = keep ? (e4[c] - a) / sd : 0.;
          for (int k = 0; k < 3; ++k)
            der[j * 12 + c * 3 + k] = keep ? dv[c * 3 + k] / sd : 0.;
        }
      }
      /* G^T R~ accumulation (se_a.py:794-843) */
      memset(xyz, 0, sizeof(double) * 4 * ng);
      for (int t = 0; t < nt; ++t) {
        const int net = m->type_one_side ? t : t * nt + ti;
        const int n0 = sec[t], nsec = sec[t + 1] - sec[t];
        if (m->compressed) {
          for (int j = 0; j < nsec; ++j) sec_x[j] = Rn[(n0 + j) * 4];
          orc_tabulate_fusion_se_a_f64(sec_out, m->table[net], m->table_info[net],
                                       sec_x, Rn + (size_t)n0 * 4, 1, nsec, ng, 1);
          for (int c = 0; c < 4; ++c)
            for (int n = 0; n < ng; ++n) xyz[c * ng + n] += sec_out[c * ng + n];
        } else {
          for (int j = n0; j < n0 + nsec; ++j) {
            emb_eval(m, net, Rn[j * 4], G, eacts);
            for (int c = 0; c < 4; ++c) {
              const double r = Rn[j * 4 + c];
              for (int n = 0; n < ng; ++n) xyz[c * ng + n] += r * G[n];
            }
          }
        }
      }
      for (int q = 0; q < 4 * ng; ++q) xyz[q] /= nnei;
      /* D = xyz^T xyz[:, :M] (se_a.py:844-850) */
      for (int n = 0; n < ng; ++n)
        for (int mm = 0; mm < M; ++mm) {
          double s = 0.;
          for (int c = 0; c < 4; ++c) s += xyz[c * ng + n] * xyz[c * ng + mm];
          D[n * M + mm] = s;
        }
      if (descriptor) memcpy(descriptor + (size_t)i * nd, D, sizeof(double) * nd);
      if (rot_mat)
        for (int n = 0; n < ng; ++n)
          for (int k = 0; k < 3; ++k)
            rot_mat[((size_t)i * ng + n) * 3 + k] = xyz[(1 + k) * ng + n];
      atom_energy[i] = fit_eval(m, ti, D, dD, facts, fhs) + m->atom_ener_bias[ti];
      /* backward: dE/dxyz */
      for (int c = 0; c < 4; ++c)
        for (int n = 0; n < ng; ++n) {
          double s = 0.;
          for (int mm = 0; mm < M; ++mm) s += dD[n * M + mm] * xyz[c * ng + mm];
          if (n < M)
            for (int n2 = 0; n2 < ng; ++n2) s += dD[n2 * M + n] * xyz[c * ng + n2];
          dxyz[c * ng + n] = s / nnei;
        }
      /* dE/dR~ per slot through the embedding (or the table) */
      for (int t = 0; t < nt; ++t) {
        const int net = m->type_one_side ? t : t * nt + ti;
        const int n0 = sec[t], nsec = sec[t + 1] - sec[t];
        if (m->compressed) {
          for (int j = 0; j < nsec; ++j) sec_x[j] = Rn[(n0 + j) * 4];
          orc_tabulate_fusion_se_a_grad_f64(sec_dx, sec_dem, m->table[net],
                                            m->table_info[net], sec_x,
                                            Rn + (size_t)n0 * 4, dxyz, 1, nsec,
                                            ng, 1);
          for (int j = 0; j < nsec; ++j) {
            for (int c = 0; c < 4; ++c) dRn[(n0 + j) * 4 + c] = sec_dem[j * 4 + c];
            dRn[(n0 + j) * 4] += sec_dx[j];
          }
        } else {
          for (int j = n0; j < n0 + nsec; ++j) {
            emb_eval(m, net, Rn[j * 4], G, eacts);
            for (int n = 0; n < ng; ++n) {
              double s = 0.;
              for (int c = 0; c < 4; ++c) s += Rn[j * 4 + c] * dxyz[c * ng + n];
              dG[n] = s;
            }
            for (int c = 0; c < 4; ++c) {
              double s = 0.;
              for (int n = 0; n < ng; ++n) s += G[n] * dxyz[c * ng + n];
              dRn[j * 4 + c] = s;
            }
            dRn[j * 4] += emb_backprop(m, net, eacts, dG);
          }
        }
      }
      /* pair gradient dE/dd_ij = -sum_c dRn[c] * der[c] (der is w.r.t. the
       * centre atom) */
      for (int j = 0; j < nnei; ++j) {
        const size_t s = (size_t)i * nnei + j;
        for (int k = 0; k < 3; ++k) {
          double g = 0.;
          for (int c = 0; c < 4; ++c) g -= dRn[j * 4 + c] * der[j * 12 + c * 3 + k];
          gpair[s * 3 + k] = nlist[s] >= 0 ? g : 0.;
        }
      }
    }
    free(Rn); free(dRn); free(der); free(xyz); free(dxyz); free(D); free(dD);
    free(G); free(dG); free(eacts); free(facts); free(fhs); free(sec_out);
    free(sec_dx); free(sec_dem); free(sec_x);
  }
  /* F = -dE/dr; virial_kl = -sum g_k d_l; atomic virial on the neighbour
   * (transform_output.py:20-99 with the atomic-virial correction) */
  memset(force_ext, 0, sizeof(double) * (size_t)nall * 3);
  memset(virial, 0, sizeof(double) * 9);
  if (atom_virial_ext) memset(atom_virial_ext, 0, sizeof(double) * (size_t)nall * 9);
  for (int i = 0; i < nloc; ++i)
    for (int j = 0; j < nnei; ++j) {
      const size_t s = (size_t)i * nnei + j;
      const int e = nlist[s];
      if (e < 0) continue;
      const double* g = gpair + s * 3;
      const double* d = dpair + s * 3;
      for (int k = 0; k < 3; ++k) {
        force_ext[(size_t)e * 3 + k] -= g[k];
        force_ext[(size_t)i * 3 + k] += g[k];
      }
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
          virial[k * 3 + l] -= g[k] * d[l];
          if (atom_virial_ext) atom_virial_ext[(size_t)e * 9 + k * 3 + l] -= g[k] * d[l];
        }
    }
  free(gpair);
  free(dpair);
  return 0;
}
