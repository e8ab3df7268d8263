// Neighbour lists: periodic wrap, ghost layout, the O(N) cell-list build in
// the reference PyTorch order, and the formatting of a candidate list in the
// reference C++ order.  Also the sorted transpose of a list used to gather
// neighbour contributions without atomics.
#include <algorithm>
#include <cmath>
#include <vector>

#include "nlist.cuh"

namespace dpgb {

// ---------------------------------------------------------------------------
// host geometry helpers
int box_geom(const double* box, CellGeom& g) {
  if (!box) return fail(DPGB_EINVAL, "box is required");
  double c[3][3];
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) c[a][b] = box[a * 3 + b];
  const double det = c[0][0] * (c[1][1] * c[2][2] - c[1][2] * c[2][1]) -
                     c[0][1] * (c[1][0] * c[2][2] - c[1][2] * c[2][0]) +
                     c[0][2] * (c[1][0] * c[2][1] - c[1][1] * c[2][0]);
  if (!(std::fabs(det) > 0)) return fail(DPGB_EINVAL, "singular box");
  double r[3][3];
  r[0][0] = (c[1][1] * c[2][2] - c[1][2] * c[2][1]) / det;
  r[0][1] = (c[0][2] * c[2][1] - c[0][1] * c[2][2]) / det;
  r[0][2] = (c[0][1] * c[1][2] - c[0][2] * c[1][1]) / det;
  r[1][0] = (c[1][2] * c[2][0] - c[1][0] * c[2][2]) / det;
  r[1][1] = (c[0][0] * c[2][2] - c[0][2] * c[2][0]) / det;
  r[1][2] = (c[0][2] * c[1][0] - c[0][0] * c[1][2]) / det;
  r[2][0] = (c[1][0] * c[2][1] - c[1][1] * c[2][0]) / det;
  r[2][1] = (c[0][1] * c[2][0] - c[0][0] * c[2][1]) / det;
  r[2][2] = (c[0][0] * c[1][1] - c[0][1] * c[1][0]) / det;
  // a diagonal cell inverts exactly to 1/L (as LU-based inversion does), so
  // the wrap of an orthorhombic box is bitwise that of the reference
  const bool diag = c[0][1] == 0 && c[0][2] == 0 && c[1][0] == 0 && c[1][2] == 0 &&
                    c[2][0] == 0 && c[2][1] == 0;
  if (diag)
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) r[a][b] = a == b ? 1.0 / c[a][a] : 0.0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      g.cell[a * 3 + b] = c[a][b];
      g.rec[a * 3 + b] = r[a][b];
    }
  g.periodic = 1;
  return DPGB_OK;
}

static void face_distances(const CellGeom& g, double face[3]) {
  const double* c = g.cell;
  auto cr = [&](int p, int q) {
    const double x = c[p * 3 + 1] * c[q * 3 + 2] - c[p * 3 + 2] * c[q * 3 + 1];
    const double y = c[p * 3 + 2] * c[q * 3 + 0] - c[p * 3 + 0] * c[q * 3 + 2];
    const double z = c[p * 3 + 0] * c[q * 3 + 1] - c[p * 3 + 1] * c[q * 3 + 0];
    return std::sqrt(x * x + y * y + z * z);
  };
  const double vol = std::fabs(c[0] * (c[4] * c[8] - c[5] * c[7]) - c[1] * (c[3] * c[8] - c[5] * c[6]) +
                               c[2] * (c[3] * c[7] - c[4] * c[6]));
  face[0] = vol / cr(1, 2);
  face[1] = vol / cr(2, 0);
  face[2] = vol / cr(0, 1);
}

// Error bound of the staged FP32 distances of a list of radius R: a stencil
// atom lies within (reach_k + 1/2) cell edges of the centre cell's centre
// along each cell vector k, so its coordinates relative to that centre are
// below m = sum_k (reach_k + 1/2) |a_k| / n_k; each is rounded to FP32
// (<= 2^-24 m, doubled for margin: u); a displacement component then errs
// by <= 2 u + 2^-24 R and the FP32 norm adds <= 2^-22 R.
static float staged_eps(const CellGeom& g, double R) {
  double m = 0.0;
  for (int k = 0; k < 3; ++k) {
    const double edge = g.periodic ? std::sqrt(g.cell[3 * k] * g.cell[3 * k] + g.cell[3 * k + 1] * g.cell[3 * k + 1] +
                                               g.cell[3 * k + 2] * g.cell[3 * k + 2]) / g.ncell[k]
                                   : g.csize[k];
    m += (g.reach[k] + 0.5) * edge;
  }
  const double u = m * 0x1p-23;
  return (float)(1.7320508075688772 * (2.0 * u + R * 0x1p-24) + R * 0x1p-22 + 1e-7);
}

int periodic_geom(const double* box, double rcut, int nshift, const int* shift_idx, CellGeom& g,
                  std::vector<int>& shift_pos) {
  DPGB_TRY(box_geom(box, g));
  if (!shift_idx || nshift <= 0) return fail(DPGB_EINVAL, "shift_idx is required with a box");
  double face[3];
  face_distances(g, face);
  const double rc_margin = rcut * (1.0 + 1e-9) + 1e-12;
  for (int d = 0; d < 3; ++d) {
    int n = (int)std::floor(face[d] / rc_margin);
    // up to 1024 cells per direction (elongated boxes keep cells near rcut)
    n = n < 1 ? 1 : (n > 1024 ? 1024 : n);
    g.ncell[d] = n;
    g.reach[d] = (int)std::ceil(rc_margin * n / face[d]);
    g.nbuff[d] = (int)std::ceil(rcut / face[d]);
  }
  // the cell list is O(cells) in memory: halve the longest direction of a
  // huge box until it holds at most 2^24 cells
  while ((long long)g.ncell[0] * g.ncell[1] * g.ncell[2] > (1LL << 24)) {
    const int d = g.ncell[0] >= g.ncell[1] && g.ncell[0] >= g.ncell[2] ? 0 : (g.ncell[1] >= g.ncell[2] ? 1 : 2);
    g.ncell[d] = (g.ncell[d] + 1) / 2;
    g.reach[d] = (int)std::ceil(rc_margin * g.ncell[d] / face[d]);
  }
  const int sx = 2 * g.nbuff[0] + 1, sy = 2 * g.nbuff[1] + 1, sz = 2 * g.nbuff[2] + 1;
  if (nshift != sx * sy * sz)
    return fail(DPGB_EINVAL, "shift_idx must enumerate the (2*nbuff+1)^3 periodic images, nbuff = ceil(rcut/face distance)");
  shift_pos.assign((size_t)sx * sy * sz, -1);
  g.zero_shift = -1;
  for (int s = 0; s < nshift; ++s) {
    const int tx = shift_idx[3 * s], ty = shift_idx[3 * s + 1], tz = shift_idx[3 * s + 2];
    if (std::abs(tx) > g.nbuff[0] || std::abs(ty) > g.nbuff[1] || std::abs(tz) > g.nbuff[2])
      return fail(DPGB_EINVAL, "shift_idx entry outside the image range");
    const int key = ((tx + g.nbuff[0]) * sy + (ty + g.nbuff[1])) * sz + (tz + g.nbuff[2]);
    if (shift_pos[key] != -1) return fail(DPGB_EINVAL, "duplicate shift in shift_idx");
    shift_pos[key] = s;
    if (tx == 0 && ty == 0 && tz == 0) g.zero_shift = s;
  }
  g.nshift = nshift;
  g.eps = staged_eps(g, rcut);
  return DPGB_OK;
}

int open_geom(const double* coord, int n, double rcut, CellGeom& g) {
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int d = 0; d < 3; ++d) {
      const double x = coord[3 * i + d];
      if (i == 0 || x < lo[d]) lo[d] = x;
      if (i == 0 || x > hi[d]) hi[d] = x;
    }
  for (int k = 0; k < 9; ++k) {
    g.cell[k] = 0;
    g.rec[k] = 0;
  }
  const double rc_margin = rcut * (1.0 + 1e-9) + 1e-12;
  for (int d = 0; d < 3; ++d) {
    const double ext = hi[d] - lo[d];
    int nc = (int)std::floor(ext / rc_margin);
    nc = nc < 1 ? 1 : (nc > 64 ? 64 : nc);
    g.ncell[d] = nc;
    g.csize[d] = std::max(ext / nc, rc_margin);
    g.origin[d] = lo[d];
    g.reach[d] = 1;
    g.nbuff[d] = 0;
  }
  g.nshift = 1;
  g.zero_shift = 0;
  g.periodic = 0;
  g.eps = staged_eps(g, rcut);
  return DPGB_OK;
}

// shift vectors t . cell (the reference's einsum over d, in order d = 0,1,2)
void shift_vectors(const CellGeom& g, const int* shift_idx, int nshift, std::vector<double>& out) {
  out.assign((size_t)nshift * 3, 0.0);
  if (!g.periodic) return;
  for (int s = 0; s < nshift; ++s)
    for (int k = 0; k < 3; ++k) {
      double v = 0.0;
      for (int d = 0; d < 3; ++d) v += (double)shift_idx[3 * s + d] * g.cell[d * 3 + k];
      out[(size_t)s * 3 + k] = v;
    }
}

int sel_from_host(const int* sel_host, int ntypes, SelInfo& s) {
  if (!sel_host || ntypes <= 0 || ntypes > DPGB_MAX_TYPES) return fail(DPGB_EINVAL, "bad sel/ntypes");
  s.ntypes = ntypes;
  s.sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) {
    if (sel_host[t] < 0) return fail(DPGB_EINVAL, "negative sel");
    s.sel[t] = sel_host[t];
    s.sec[t + 1] = s.sec[t] + sel_host[t];
  }
  s.nnei = s.sec[ntypes];
  s.strict = 0;
  s.flat = 0;
  return DPGB_OK;
}

namespace {

__device__ __forceinline__ double dist_fma(double dx, double dy, double dz) {
  // the FMA chain of torch.linalg.norm (sqrt(fma(z,z,fma(y,y,x*x)))), so
  // that near-equal distances order exactly as in the reference
  return sqrt(fma(dz, dz, fma(dy, dy, dx * dx)));
}

// wrap a point into the periodic cell (fractional coordinates mod 1), the
// arithmetic of deepmd/pt/utils/region.py:86-105
__device__ __forceinline__ void wrap_point(const double* in, const CellGeom& g, double* out) {
  const double x = in[0], y = in[1], z = in[2];
  double f[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double v = fma(z, g.rec[6 + k], fma(y, g.rec[3 + k], x * g.rec[k]));
    v = v - floor(v);
    f[k] = v;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = fma(f[2], g.cell[6 + k], fma(f[1], g.cell[3 + k], f[0] * g.cell[k]));
}

__global__ void normalize_kernel(double* __restrict__ out, const double* __restrict__ in, int n,
                                 CellGeom g, int* __restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flag_nonfinite(in + 3 * i, i, status);
  wrap_point(in + 3 * i, g, out + 3 * i);
}

__global__ void extend_kernel(double* __restrict__ cext, int* __restrict__ text,
                              int* __restrict__ mapping, const double* __restrict__ coord,
                              const int* __restrict__ atype, int nloc, int nshift,
                              const double* __restrict__ svec) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nloc * nshift) return;
  const int s = (int)(q / nloc), j = (int)(q % nloc);
#pragma unroll
  for (int k = 0; k < 3; ++k) cext[3 * q + k] = coord[3 * j + k] + svec[3 * s + k];
  if (text) text[q] = atype[j];
  if (mapping) mapping[q] = j;
}

__global__ void cell_count_kernel(int* __restrict__ cell_of, int* __restrict__ counts,
                                  const double* __restrict__ coord, int n, CellGeom g,
                                  const int* __restrict__ gate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || (gate && !gate[0])) return;
  int c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double f;
    if (g.periodic)
      f = (coord[3 * i] * g.rec[k] + coord[3 * i + 1] * g.rec[3 + k] +
           coord[3 * i + 2] * g.rec[6 + k]) * g.ncell[k];
    else
      f = (coord[3 * i + k] - g.origin[k]) / g.csize[k];
    int ci = (int)floor(f);
    ci = ci < 0 ? 0 : (ci >= g.ncell[k] ? g.ncell[k] - 1 : ci);
    c[k] = ci;
  }
  const int id = (c[0] * g.ncell[1] + c[1]) * g.ncell[2] + c[2];
  cell_of[i] = id;
  atomicAdd(&counts[id], 1);
}

__global__ void cell_fill_kernel(int* __restrict__ cell_atoms, int* __restrict__ cursor,
                                 const int* __restrict__ offsets, const int* __restrict__ cell_of,
                                 int n, const int* __restrict__ gate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || (gate && !gate[0])) return;
  const int c = cell_of[i];
  cell_atoms[offsets[c] + atomicAdd(&cursor[c], 1)] = i;
}

constexpr int kSearchWarps = 2;

// stencil cell -> (wrapped cell, periodic image); false when outside an open box
__device__ __forceinline__ bool wrap_cell(int x, int n, int periodic, int& xw, int& t) {
  if (!periodic) {
    xw = x;
    t = 0;
    return x >= 0 && x < n;
  }
  t = x >= 0 ? x / n : -((-x + n - 1) / n);
  xw = x - t * n;
  return true;
}
constexpr int kCap = 1024;

struct Cand {
  double r;
  int idx;
  int type;
};

// (distance, extended index) order.  Distances are >= +0, so their IEEE bit
// patterns order exactly like the values: the comparison runs as 64-bit
// integer compares instead of on the (narrow) FP64 pipe.
__device__ __forceinline__ bool cand_less(double ra, int ia, double rb, int ib) {
  const long long a = __double_as_longlong(ra), b = __double_as_longlong(rb);
  return a < b || (a == b && ia < ib);
}

// Placement of one ranked pair: per type (the first sel[t] of its type among
// the global top sum(sel)) or, for flat candidate rows, at its global rank.
// A strict list records the width a missing slot would have needed.
__device__ __forceinline__ void place_pair(int* __restrict__ row, int rank, int trank, int t, int e,
                                           const SelInfo& sel, int* __restrict__ status) {
  if (sel.flat) {
    if (rank < sel.nnei)
      row[rank] = e;
    else if (sel.strict)
      atomicMax(&status[kStatusTruncated], rank + 1);
  } else if (rank < sel.nnei && t < sel.ntypes && trank < sel.sel[t]) {
    row[sel.sec[t] + trank] = e;
  } else if (sel.strict) {
    atomicMax(&status[kStatusTruncated], trank + 1);
  }
}

// One warp per centre atom: gather the atoms of the stencil cells within
// rcut, rank them by (distance, extended index), keep the nearest nsel and
// place each in its type section while its per-type rank < sel[t].
__global__ void __launch_bounds__(kSearchWarps * 32)
nlist_pt_kernel(int* __restrict__ nlist, const double* __restrict__ coord,
                const int* __restrict__ atype, const int* __restrict__ cell_of,
                const int* __restrict__ offsets, const int* __restrict__ cell_atoms,
                const int* __restrict__ shift_pos, const double* __restrict__ svec, int nloc,
                CellGeom g, double rcut, SelInfo sel, const int* __restrict__ only_cells,
                int* __restrict__ status, const int* __restrict__ gate) {
  __shared__ double s_r[kSearchWarps][kCap];
  __shared__ int s_idx[kSearchWarps][kCap];
  __shared__ int s_type[kSearchWarps][kCap];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (gate && !gate[0]) return;
  // as the fallback of the staged kernel: nothing to do unless some cell was
  // flagged (only_cells[ncell] is set with any flag)
  if (only_cells && !only_cells[g.ncell[0] * g.ncell[1] * g.ncell[2]]) return;
  // atoms in a grid-stride loop: as the fallback, most atoms only check their
  // cell's flag
  for (int i = blockIdx.x * kSearchWarps + warp; i < nloc; i += gridDim.x * kSearchWarps) {
  if (only_cells && !only_cells[cell_of[i]]) continue;  // handled by the staged kernel
  __syncwarp();  // the previous atom's reads of s_r / s_idx / s_type are done
  int* row = nlist + (size_t)i * sel.nnei;
  for (int q = lane; q < sel.nnei; q += 32) row[q] = -1;
  if (atype[i] < 0) continue;
  const double xi = coord[3 * i], yi = coord[3 * i + 1], zi = coord[3 * i + 2];
  const int ci = cell_of[i];
  const int cz = ci % g.ncell[2], cy = (ci / g.ncell[2]) % g.ncell[1],
            cx = ci / (g.ncell[1] * g.ncell[2]);
  const int sy = 2 * g.nbuff[1] + 1, sz = 2 * g.nbuff[2] + 1;
  int n = 0;
  bool overflow = false;
  for (int ox = -g.reach[0]; ox <= g.reach[0]; ++ox) {
    int xw, tx;
    if (!wrap_cell(cx + ox, g.ncell[0], g.periodic, xw, tx)) continue;
    for (int oy = -g.reach[1]; oy <= g.reach[1]; ++oy) {
      int yw, ty;
      if (!wrap_cell(cy + oy, g.ncell[1], g.periodic, yw, ty)) continue;
      for (int oz = -g.reach[2]; oz <= g.reach[2]; ++oz) {
        int zw, tz;
        if (!wrap_cell(cz + oz, g.ncell[2], g.periodic, zw, tz)) continue;
        if (abs(tx) > g.nbuff[0] || abs(ty) > g.nbuff[1] || abs(tz) > g.nbuff[2]) continue;
        const int s = shift_pos[((tx + g.nbuff[0]) * sy + (ty + g.nbuff[1])) * sz + (tz + g.nbuff[2])];
        const double sx0 = svec[3 * s], sx1 = svec[3 * s + 1], sx2 = svec[3 * s + 2];
        const int c = (xw * g.ncell[1] + yw) * g.ncell[2] + zw;
        const int beg = offsets[c], end = offsets[c + 1];
        for (int p0 = beg; p0 < end; p0 += 32) {
          const int p = p0 + lane;
          bool keep = false;
          double r = 0.0;
          int j = -1, tj = -1;
          if (p < end) {
            j = cell_atoms[p];
            tj = atype[j];
            if (tj >= 0 && !(j == i && s == g.zero_shift)) {
              const double dx = (coord[3 * j] + sx0) - xi;
              const double dy = (coord[3 * j + 1] + sx1) - yi;
              const double dz = (coord[3 * j + 2] + sx2) - zi;
              r = dist_fma(dx, dy, dz);
              keep = r <= rcut;
            }
          }
          const unsigned m = __ballot_sync(0xffffffffu, keep);
          const int pos = n + __popc(m & ((1u << lane) - 1u));
          if (keep) {
            if (pos < kCap) {
              s_r[warp][pos] = r;
              s_idx[warp][pos] = s * nloc + j;
              s_type[warp][pos] = tj;
            } else {
              overflow = true;
            }
          }
          n += __popc(m);
        }
      }
    }
  }
  overflow = __any_sync(0xffffffffu, overflow);
  if (overflow) {
    if (lane == 0) {
      atomicMax(&status[kStatusOverflow], n);
      atomicMax(&status[kStatusOverflowAtom], i + 1);
    }
    continue;
  }
  __syncwarp();
  for (int k = lane; k < n; k += 32) {
    const double rk = s_r[warp][k];
    const int ik = s_idx[warp][k], tk = s_type[warp][k];
    int rank = 0, trank = 0;
    for (int m2 = 0; m2 < n; ++m2) {
      const bool lt = cand_less(s_r[warp][m2], s_idx[warp][m2], rk, ik);
      rank += lt;
      trank += lt && s_type[warp][m2] == tk;
    }
    // topk(sum(sel)): candidates of global rank >= nnei are dropped
    place_pair(row, rank, trank, tk, ik, sel, status);
  }
  }
}

// Staged form of nlist_pt_kernel: one CTA per cell.  The atoms of the cell's
// 27 stencil cells are copied once into shared memory (image-shifted
// coordinates, extended index, type), so the cell's centre atoms (one warp
// each) scan them without global gathers.  Same distances (the FMA norm of
// (r_j + shift) - r_i), same ranking by (distance, extended index), same
// per-type placement: the list is bitwise that of nlist_pt_kernel.  A cell
// whose stencil holds more than stage_cap atoms is flagged and left to
// nlist_pt_kernel.
constexpr int kCellWarps = 8;   // warps of nlist_cell_kernel (four CTAs, 32 warps per SM)
constexpr int kBatchWarps = 4;  // warps of nlist_cell_batch_kernel
constexpr int kKeptCap = 512;  // per-warp kept pairs of the skin selection (at most)
// Shared memory of the staged kernels: stage_cap stencil atoms (3 floats, 2
// ints) and, for typed lists, kept_cap pairs per warp (a double key, 2 ints).
// Typed lists stage 1536 atoms and keep 192 pairs per warp (55 KB: four
// CTAs per SM) unless the mean density asks for more (typed_kept_cap);
// flat candidate rows keep none and stage 2688 (a stencil at rcut + skin).
constexpr int kTypedStageCap = 1536, kTypedKeptMin = 192, kTypedKeptMax = 384, kFlatStageCap = 2688;

// Kept pairs per warp for typed lists: 1.5 x the mean count within rcut
// (the atoms' mean density) + 48, in [192, 384].  An atom with more
// candidates sends its cell to nlist_pt_kernel.
int typed_kept_cap(const CellGeom& g, int nloc, double rcut) {
  double vol;
  if (g.periodic) {
    const double* c = g.cell;
    vol = std::fabs(c[0] * (c[4] * c[8] - c[5] * c[7]) - c[1] * (c[3] * c[8] - c[5] * c[6]) +
                    c[2] * (c[3] * c[7] - c[4] * c[6]));
  } else {
    vol = g.csize[0] * g.csize[1] * g.csize[2] * g.ncell[0] * g.ncell[1] * g.ncell[2];
  }
  const double mean = vol > 0 ? nloc / vol * (4.0 / 3.0) * 3.141592653589793 * rcut * rcut * rcut : 0.0;
  const double want = 1.5 * mean + 48.0;
  const int cap = want >= kTypedKeptMax ? kTypedKeptMax : ((int)want + 31) / 32 * 32;
  return cap < kTypedKeptMin ? kTypedKeptMin : cap;
}

size_t cell_stage_smem(int stage_cap, int kept_cap) {
  return (size_t)stage_cap * (3 * sizeof(float) + 2 * sizeof(int)) +
         (size_t)kCellWarps * kept_cap * (sizeof(double) + 2 * sizeof(int));
}

// Rank a warp's kept list by exact FP64 distance, then extended index, and
// place it.  Each lane holds up to four kept entries in registers and
// streams the list once per 128.
__device__ void staged_rank_place(int* __restrict__ row, const double* __restrict__ wr, const int* __restrict__ wi,
                                  const int* __restrict__ wt, int n, const SelInfo& sel, int lane,
                                  int* __restrict__ status) {
  for (int k0 = 0; k0 < n; k0 += 128) {
    long long rk[4];
    int ik[4], tk[4], rank[4], trank[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = k0 + lane + 32 * q;
      rk[q] = k < n ? __double_as_longlong(wr[k]) : 0x7fffffffffffffffLL;
      ik[q] = k < n ? wi[k] : 0x7fffffff;
      tk[q] = k < n ? wt[k] : -1;
      rank[q] = trank[q] = 0;
    }
    for (int m2 = 0; m2 < n; ++m2) {
      const long long rm = __double_as_longlong(wr[m2]);
      const int im = wi[m2], tm = wt[m2];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const bool lt = rm < rk[q] || (rm == rk[q] && im < ik[q]);
        rank[q] += lt;
        trank[q] += lt && tm == tk[q];
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (k0 + lane + 32 * q < n) place_pair(row, rank[q], trank[q], tk[q], ik[q], sel, status);
  }
}

// The same ranking on FP32 distances wf that lie within eps of the exact
// FP64 ones.  Two keys closer than tie = 2 eps (or equal) may order
// differently in FP64: then nothing of that group is placed and it returns
// true (the caller redoes the atom in FP64 and clears the row first).
__device__ bool rank_place_f32(int* __restrict__ row, const float* __restrict__ wf, const int* __restrict__ wi,
                               const int* __restrict__ wt, int n, float tie, const SelInfo& sel, int lane,
                               int* __restrict__ status) {
  for (int k0 = 0; k0 < n; k0 += 128) {
    float rk[4];
    int ik[4], tk[4], rank[4], trank[4];
    bool near = false;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = k0 + lane + 32 * q;
      rk[q] = k < n ? wf[k] : __int_as_float(0x7f800000);
      ik[q] = k < n ? wi[k] : 0x7fffffff;
      tk[q] = k < n ? wt[k] : -1;
      rank[q] = trank[q] = 0;
    }
    for (int m2 = 0; m2 < n; ++m2) {
      const float rm = wf[m2];
      const int im = wi[m2], tm = wt[m2];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const bool lt = rm < rk[q] || (rm == rk[q] && im < ik[q]);
        rank[q] += lt;
        trank[q] += lt && tm == tk[q];
        near |= im != ik[q] && fabsf(rm - rk[q]) <= tie;
      }
    }
    if (__any_sync(0xffffffffu, near)) return true;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (k0 + lane + 32 * q < n) place_pair(row, rank[q], trank[q], tk[q], ik[q], sel, status);
  }
  return false;
}

__device__ __forceinline__ bool key_less(float ka, int ea, float kb, int eb) {
  return ka < kb || (ka == kb && ea < eb);
}

// Warp-wide bitonic sort of 128 (key, index, type) triples, element
// 32 q + lane in register q of each lane, ascending by (key, index).
// Partners closer than 32 are exchanged by shuffles, those 32 or 64 apart
// sit in the same lane's registers.
__device__ __forceinline__ void warp_sort128(float k[4], int e[4], int t[4], int lane) {
#pragma unroll
  for (int size = 2; size <= 128; size <<= 1) {
#pragma unroll
    for (int j = size >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const int qj = j >> 5;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int p = q ^ qj;
          if (p > q) {
            const bool up = ((q * 32 + lane) & size) == 0;
            const bool sw = up ? key_less(k[p], e[p], k[q], e[q]) : key_less(k[q], e[q], k[p], e[p]);
            if (sw) {
              const float tk = k[q];
              const int te = e[q], tt = t[q];
              k[q] = k[p];
              e[q] = e[p];
              t[q] = t[p];
              k[p] = tk;
              e[p] = te;
              t[p] = tt;
            }
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float ok = __shfl_xor_sync(0xffffffffu, k[q], j);
          const int oe = __shfl_xor_sync(0xffffffffu, e[q], j);
          const int ot = __shfl_xor_sync(0xffffffffu, t[q], j);
          const int idx = q * 32 + lane;
          const bool up = (idx & size) == 0, lower = (idx & j) == 0;
          const bool o_less = key_less(ok, oe, k[q], e[q]);
          if (lower == up ? o_less : !o_less) {
            k[q] = ok;
            e[q] = oe;
            t[q] = ot;
          }
        }
      }
    }
  }
}

// Exact FP64 distance from the centre atom (xi, yi, zi) of the atom with
// extended index e = s * nloc + j (atom a_beg + j, shift vector s), as the
// exact path (exact_keep) computes it.
struct ExactDist {
  const double* coord;
  const double* svec;
  int nloc, a_beg;
  double xi, yi, zi;
  __device__ __forceinline__ double operator()(int e) const {
    const int s = e / nloc, j = a_beg + (e - s * nloc);
    return dist_fma((coord[3 * j] + svec[3 * s]) - xi, (coord[3 * j + 1] + svec[3 * s + 1]) - yi,
                    (coord[3 * j + 2] + svec[3 * s + 2]) - zi);
  }
};

// bit p of a 128-bit mask held as four words
__device__ __forceinline__ bool bit128(const unsigned (&w)[4], int p) {
  const int q = p >> 5;
  const unsigned v = q == 0 ? w[0] : (q == 1 ? w[1] : (q == 2 ? w[2] : w[3]));
  return (v >> (p & 31)) & 1u;
}

// Warp-wide bitonic sort of 32 R (key, index) pairs, element 32 q + lane in
// register q of each lane, ascending by (key, index).
template <int R>
__device__ __forceinline__ void warp_sort_kv(float (&k)[R], int (&e)[R], int lane) {
#pragma unroll
  for (int size = 2; size <= 32 * R; size <<= 1) {
#pragma unroll
    for (int j = size >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
#pragma unroll
        for (int q = 0; q < R; ++q) {
          const int p = q ^ (j >> 5);
          if (p > q) {
            const bool up = ((q * 32 + lane) & size) == 0;
            const bool sw = up ? key_less(k[p], e[p], k[q], e[q]) : key_less(k[q], e[q], k[p], e[p]);
            if (sw) {
              const float tk = k[q];
              const int te = e[q];
              k[q] = k[p];
              e[q] = e[p];
              k[p] = tk;
              e[p] = te;
            }
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < R; ++q) {
          const float ok = __shfl_xor_sync(0xffffffffu, k[q], j);
          const int oe = __shfl_xor_sync(0xffffffffu, e[q], j);
          const int idx = q * 32 + lane;
          const bool up = (idx & size) == 0, lower = (idx & j) == 0;
          const bool o_less = key_less(ok, oe, k[q], e[q]);
          if (lower == up ? o_less : !o_less) {
            k[q] = ok;
            e[q] = oe;
          }
        }
      }
    }
  }
}

// One type's kept pairs, compacted to the front of (wf, wi) (c <= 32 R of
// them): warp sort by (FP32 key, index), runs of keys within tie re-ranked
// by exact FP64 distance as in sort_place_f32, then placed by their rank
// within the type.
template <int R>
__device__ void sort_place_type(int* __restrict__ row, double* __restrict__ wr, int* __restrict__ wi, int c, int t,
                                float tie, const ExactDist& exact, const SelInfo& sel, int lane,
                                int* __restrict__ status) {
  const float* wf = reinterpret_cast<const float*>(wr);
  float k[R];
  int e[R];
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int idx = q * 32 + lane;
    k[q] = idx < c ? wf[idx] : __int_as_float(0x7f800000);
    e[q] = idx < c ? wi[idx] : 0x7fffffff;
  }
  warp_sort_kv<R>(k, e, lane);
  unsigned near[4] = {0u, 0u, 0u, 0u};  // bit p: sorted positions p and p + 1 are within tie
#pragma unroll
  for (int q = 0; q < R; ++q) {
    float next = __shfl_down_sync(0xffffffffu, k[q], 1);
    const float first_next = __shfl_sync(0xffffffffu, k[q < R - 1 ? q + 1 : q], 0);
    if (lane == 31) next = first_next;
    const int idx = q * 32 + lane;
    near[q] = __ballot_sync(0xffffffffu, idx + 1 < c && next - k[q] <= tie);
  }
  if (near[0] | near[1] | near[2] | near[3]) {
    __syncwarp();  // every lane has read its FP32 key before wr is overwritten
    bool member[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int p = q * 32 + lane;
      member[q] = bit128(near, p) || (p > 0 && bit128(near, p - 1));
      wi[p] = e[q];
      if (member[q]) wr[p] = exact(e[q]);
    }
    __syncwarp();
    int np[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      const int p = q * 32 + lane;
      np[q] = p;
      if (member[q]) {
        int lo = p, hi = p;
        while (lo > 0 && bit128(near, lo - 1)) --lo;
        while (bit128(near, hi)) ++hi;  // a near bit needs p + 1 < c <= 32 R
        const double r = wr[p];
        int cnt = 0;
        for (int m = lo; m <= hi; ++m) {
          const double rm = wr[m];
          cnt += rm < r || (rm == r && wi[m] < e[q]);
        }
        np[q] = lo + cnt;
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < R; ++q)
      if (member[q]) wi[np[q]] = e[q];
    __syncwarp();
#pragma unroll
    for (int q = 0; q < R; ++q) e[q] = wi[q * 32 + lane];
  }
#pragma unroll
  for (int q = 0; q < R; ++q) {
    const int idx = q * 32 + lane;
    if (idx < c) place_pair(row, 0, idx, t, e[q], sel, status);
  }
}

// The kept pairs (k, e, t: element 32 q + lane in register q), sorted and
// placed one type at a time when that gives the same list as the global
// ranking: no more pairs than sum(sel) (so the global cut keeps all) and at
// most 64 of each type.  Sorting each type's few dozen pairs costs less than
// one 128-wide sort.  Returns false (nothing written) otherwise.
__device__ bool sort_place_by_type(int* __restrict__ row, double* __restrict__ wr, int* __restrict__ wi,
                                   const float (&k)[4], const int (&e)[4], const int (&tt)[4], int n, float tie,
                                   const ExactDist& exact, const SelInfo& sel, int lane,
                                   int* __restrict__ status) {
  if (n > sel.nnei) return false;
  int total = 0;
  bool fits = true;
  for (int t = 0; t < sel.ntypes; ++t) {
    int c = 0;
#pragma unroll
    for (int q = 0; q < 4; ++q) c += __popc(__ballot_sync(0xffffffffu, tt[q] == t && q * 32 + lane < n));
    total += c;
    fits = fits && c <= 64;
  }
  if (!fits || total != n) return false;
  float* wf = reinterpret_cast<float*>(wr);
  const unsigned below = (1u << lane) - 1u;
  for (int t = 0; t < sel.ntypes; ++t) {
    __syncwarp();  // the previous type's reads of (wf, wi) are done
    int base = 0;  // ends as the type's count
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool mine = tt[q] == t && q * 32 + lane < n;
      const unsigned m = __ballot_sync(0xffffffffu, mine);
      if (mine) {
        wf[base + __popc(m & below)] = k[q];
        wi[base + __popc(m & below)] = e[q];
      }
      base += __popc(m);
    }
    __syncwarp();
    if (base == 0) continue;
    if (base <= 32)
      sort_place_type<1>(row, wr, wi, base, t, tie, exact, sel, lane, status);
    else
      sort_place_type<2>(row, wr, wi, base, t, tie, exact, sel, lane, status);
  }
  return true;
}

// Placement of up to 128 kept pairs with FP32 keys (the first floats of wr,
// within eps of the exact distances) through a warp sort: the sorted
// position is the global rank, same-type lanes of each 32-chunk
// (match_any) plus the running count of their type (s_base, per warp) give
// the rank within the type.  Neighbours in the sorted order whose keys are
// closer than tie = 2 eps (or equal) may order differently in FP64; each
// maximal run of such positions is re-ranked by exact (distance, extended
// index), which leaves the order that of the exact ranking: a key more than
// 2 eps below another has the smaller exact distance.
__device__ void sort_place_f32(int* __restrict__ row, double* __restrict__ wr, int* __restrict__ wi,
                               int* __restrict__ wt, int n, float tie, const ExactDist& exact, const SelInfo& sel,
                               int lane, int* __restrict__ status, int* __restrict__ s_base) {
  const float* wf = reinterpret_cast<const float*>(wr);
  float k[4];
  int e[4], t[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int idx = q * 32 + lane;
    k[q] = idx < n ? wf[idx] : __int_as_float(0x7f800000);
    e[q] = idx < n ? wi[idx] : 0x7fffffff;
    t[q] = idx < n ? wt[idx] : -1;
  }
  if (sort_place_by_type(row, wr, wi, k, e, t, n, tie, exact, sel, lane, status)) return;
  warp_sort128(k, e, t, lane);
  unsigned near[4];  // bit p: sorted positions p and p + 1 are within tie
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float next = __shfl_down_sync(0xffffffffu, k[q], 1);
    const float first_next = __shfl_sync(0xffffffffu, k[q < 3 ? q + 1 : q], 0);
    if (lane == 31) next = first_next;
    const int idx = q * 32 + lane;
    near[q] = __ballot_sync(0xffffffffu, idx + 1 < n && next - k[q] <= tie);
  }
  if (near[0] | near[1] | near[2] | near[3]) {
    __syncwarp();  // every lane has read its FP32 key before wr is overwritten
    bool member[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int p = q * 32 + lane;
      member[q] = bit128(near, p) || (p > 0 && bit128(near, p - 1));
      wi[p] = e[q];
      wt[p] = t[q];
      if (member[q]) wr[p] = exact(e[q]);
    }
    __syncwarp();
    int np[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int p = q * 32 + lane;
      np[q] = p;
      if (member[q]) {
        int lo = p, hi = p;
        while (lo > 0 && bit128(near, lo - 1)) --lo;
        while (bit128(near, hi)) ++hi;  // a near bit needs p + 1 < n <= 128
        const double r = wr[p];
        int c = 0;
        for (int m = lo; m <= hi; ++m) {
          const double rm = wr[m];
          c += rm < r || (rm == r && wi[m] < e[q]);
        }
        np[q] = lo + c;
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (member[q]) {
        wi[np[q]] = e[q];
        wt[np[q]] = t[q];
      }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int p = q * 32 + lane;
      e[q] = wi[p];
      t[q] = wt[p];
    }
  }
  if (lane < sel.ntypes) s_base[lane] = 0;
  __syncwarp();
  const unsigned below = (1u << lane) - 1u;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int tq = t[q];
    const unsigned m = __match_any_sync(0xffffffffu, tq);
    const int tr = (tq >= 0 ? s_base[tq] : 0) + __popc(m & below);
    __syncwarp();
    if (tq >= 0 && lane == __ffs(m) - 1) s_base[tq] += __popc(m);
    __syncwarp();
    const int idx = q * 32 + lane;
    if (idx < n) place_pair(row, idx, tr, tq, e[q], sel, status);
  }
}

// Exact FP64 distances of a warp's packed candidates (extended indices wi,
// e = s * nloc + j, types wt; atom j is a_beg + j): those with r <= rcut are
// packed again, in place, as (wr, wi, wt).  The FP64 pipe is narrow on this
// part, so it runs only on full warps of packed candidates.
__device__ int exact_keep(double* __restrict__ wr, int* __restrict__ wi, int* __restrict__ wt, int nc,
                          const double* __restrict__ coord, const double* __restrict__ svec, int nloc, int a_beg,
                          double xi, double yi, double zi, double rcut, int lane) {
  const unsigned below = (1u << lane) - 1u;
  int n = 0;
  for (int k0 = 0; k0 < nc; k0 += 32) {
    const int k = k0 + lane;
    bool keep = false;
    double r = 0.0;
    int e = 0, t = 0;
    if (k < nc) {
      e = wi[k];
      t = wt[k];
      const int s = e / nloc, j = a_beg + (e - s * nloc);
      const double dx = (coord[3 * j] + svec[3 * s]) - xi;
      const double dy = (coord[3 * j + 1] + svec[3 * s + 1]) - yi;
      const double dz = (coord[3 * j + 2] + svec[3 * s + 2]) - zi;
      r = dist_fma(dx, dy, dz);
      keep = r <= rcut;
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    __syncwarp();  // every lane has read its slot before any is overwritten
    const int pos = n + __popc(m & below);  // pos <= k: never a slot still to be read
    if (keep) {
      wr[pos] = r;
      wi[pos] = e;
      wt[pos] = t;
    }
    n += __popc(m);
  }
  __syncwarp();
  return n;
}

// centre of cell (cx, cy, cz)
__device__ __forceinline__ void cell_centre(const CellGeom& g, int cx, int cy, int cz, double o[3]) {
  if (g.periodic) {
    const double f0 = (cx + 0.5) / g.ncell[0], f1 = (cy + 0.5) / g.ncell[1], f2 = (cz + 0.5) / g.ncell[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = f0 * g.cell[k] + f1 * g.cell[3 + k] + f2 * g.cell[6 + k];
  } else {
    o[0] = g.origin[0] + (cx + 0.5) * g.csize[0];
    o[1] = g.origin[1] + (cy + 0.5) * g.csize[1];
    o[2] = g.origin[2] + (cz + 0.5) * g.csize[2];
  }
}

// One centre atom against the staged stencil atoms (FP32 coordinates
// relative to the cell centre), one warp, writing its row:
// * flat candidate rows (sel.flat): every staged atom within rcut + eps, in
//   staging order, no distances beyond FP32;
// * typed lists: FP32 distances within eps of the exact ones decide the
//   cutoff and the order; an atom with a distance within eps of rcut or two
//   within 2 eps of each other is redone in exact FP64 — so the list is
//   always that of the exact (distance, extended index) ranking.
// Returns 0, or -(candidates) - 1 when more than kept_cap candidates (typed
// lists; the row is then incomplete).
__device__ int staged_list_atom(int* __restrict__ row, double* __restrict__ wr, int* __restrict__ wi,
                                int* __restrict__ wt, const float4* __restrict__ s4, const int* __restrict__ sidx,
                                int total, int self, float xf, float yf, float zf,
                                float eps, const double* __restrict__ coord, const double* __restrict__ svec,
                                int nloc, int a_beg, double xi, double yi, double zi, double rcut, const SelInfo& sel,
                                int lane, int* __restrict__ status, int* __restrict__ s_base, int kept_cap) {
  const unsigned below = (1u << lane) - 1u;
  const float rin = (float)rcut - eps, rout = (float)rcut + eps;
  const float rout2 = rout * rout;
  if (sel.flat) {
    int nc = 0;
    for (int p0 = 0; p0 < total; p0 += 32) {
      const int p = p0 + lane;
      bool cand = false;
      if (p < total) {
        const float4 q = s4[p];  // x, y, z, type bits
        const float fx = q.x - xf, fy = q.y - yf, fz = q.z - zf;
        const float d2 = fx * fx + fy * fy + fz * fz;
        // the atom itself (zero image) is the one entry at distance exactly 0
        cand = __float_as_int(q.w) >= 0 && d2 <= rout2 && !(d2 == 0.f && sidx[p] == self);
      }
      const unsigned m = __ballot_sync(0xffffffffu, cand);
      const int pos = nc + __popc(m & below);
      if (cand && pos < sel.nnei) row[pos] = sidx[p];
      nc += __popc(m);
    }
    if (nc > sel.nnei && sel.strict && lane == 0) atomicMax(&status[kStatusTruncated], nc);
    return 0;
  }
  float* wf = reinterpret_cast<float*>(wr);  // FP32 keys (first half of the FP64 key buffer)
  int nc = 0;
  bool band = false;
  for (int p0 = 0; p0 < total; p0 += 32) {
    const int p = p0 + lane;
    bool cand = false;
    float r = 0.f;
    int tq = -1;
    if (p < total) {
      const float4 q = s4[p];  // x, y, z, type bits
      tq = __float_as_int(q.w);
      const float fx = q.x - xf, fy = q.y - yf, fz = q.z - zf;
      const float d2 = fx * fx + fy * fy + fz * fz;
      // the atom itself (zero image) is the one entry at distance exactly 0
      if (tq >= 0 && d2 <= rout2 && !(d2 == 0.f && sidx[p] == self)) {
        cand = true;
        r = sqrtf(d2);
        band |= r > rin;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, cand);
    const int pos = nc + __popc(m & below);
    if (cand && pos < kept_cap) {
      wf[pos] = r;
      wi[pos] = sidx[p];
      wt[pos] = tq;
    }
    nc += __popc(m);
  }
  if (nc > kept_cap) return -nc - 1;
  band = __any_sync(0xffffffffu, band);
  __syncwarp();
  if (!band) {
    if (nc <= 128) {
      sort_place_f32(row, wr, wi, wt, nc, 2.f * eps, ExactDist{coord, svec, nloc, a_beg, xi, yi, zi}, sel, lane,
                     status, s_base);
      return 0;
    }
    if (!rank_place_f32(row, wf, wi, wt, nc, 2.f * eps, sel, lane, status)) return 0;
  }
  // exact FP64: clear what the FP32 pass may have placed, then rank exactly
  if (lane == 0) atomicAdd(&status[kStatusExact], 1);
  __syncwarp();
  for (int q = lane; q < sel.nnei; q += 32) row[q] = -1;
  __syncwarp();
  const int n = exact_keep(wr, wi, wt, nc, coord, svec, nloc, a_beg, xi, yi, zi, rcut, lane);
  staged_rank_place(row, wr, wi, wt, n, sel, lane, status);
  return 0;
}

__global__ void __launch_bounds__(kCellWarps * 32, 4)
nlist_cell_kernel(int* __restrict__ nlist, const double* __restrict__ coord, const int* __restrict__ atype,
                  const int* __restrict__ offsets, const int* __restrict__ cell_atoms,
                  const int* __restrict__ shift_pos, const double* __restrict__ svec, int nloc, CellGeom g,
                  double rcut, SelInfo sel, int* __restrict__ fallback, int* __restrict__ status,
                  const int* __restrict__ gate, int stage_cap, int kept_cap) {
  if (gate && !gate[0]) return;
  extern __shared__ __align__(16) unsigned char smem[];
  double* kr = reinterpret_cast<double*>(smem);
  float4* s4 = reinterpret_cast<float4*>(kr + kCellWarps * kept_cap);  // staged x, y, z, type bits
  int* sidx = reinterpret_cast<int*>(s4 + stage_cap);
  int* kidx = sidx + stage_cap;
  int* ktype = kidx + kCellWarps * kept_cap;
  __shared__ int s_cell[27], s_shift[27], s_off[28];
  __shared__ int s_tb[kCellWarps][DPGB_MAX_TYPES];  // per-type running counts of sort_place_f32
  __shared__ double s_oc[3];
  const int c = blockIdx.x, tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int cz = c % g.ncell[2], cy = (c / g.ncell[2]) % g.ncell[1], cx = c / (g.ncell[1] * g.ncell[2]);
  const int sy_ = 2 * g.nbuff[1] + 1, sz_ = 2 * g.nbuff[2] + 1;
  if (tid < 27) {
    const int ox = tid / 9 - 1, oy = (tid / 3) % 3 - 1, oz = tid % 3 - 1;
    int xw, tx, yw, ty, zw, tz;
    bool ok = wrap_cell(cx + ox, g.ncell[0], g.periodic, xw, tx) && wrap_cell(cy + oy, g.ncell[1], g.periodic, yw, ty) &&
              wrap_cell(cz + oz, g.ncell[2], g.periodic, zw, tz);
    ok = ok && abs(tx) <= g.nbuff[0] && abs(ty) <= g.nbuff[1] && abs(tz) <= g.nbuff[2];
    s_cell[tid] = ok ? (xw * g.ncell[1] + yw) * g.ncell[2] + zw : -1;
    s_shift[tid] = ok ? shift_pos[((tx + g.nbuff[0]) * sy_ + (ty + g.nbuff[1])) * sz_ + (tz + g.nbuff[2])] : 0;
  }
  __syncthreads();
  if (tid == 0) {
    s_off[0] = 0;
    for (int k = 0; k < 27; ++k)
      s_off[k + 1] = s_off[k] + (s_cell[k] >= 0 ? offsets[s_cell[k] + 1] - offsets[s_cell[k]] : 0);
  }
  __syncthreads();
  const int total = s_off[27];
  if (total > stage_cap) {  // left to nlist_pt_kernel
    if (tid == 0) fallback[c] = fallback[gridDim.x] = 1;  // [ncell]: some cell is flagged
    return;
  }
  // FP32 copies relative to the centre cell's centre (magnitudes within 1.5
  // cell diagonals: the rounding bound g.eps)
  if (tid == 0) cell_centre(g, cx, cy, cz, s_oc);
  __syncthreads();
  const double ox = s_oc[0], oy = s_oc[1], oz = s_oc[2];
  const float eps = g.eps;
  for (int q = tid; q < total; q += blockDim.x) {
    int k = 0;
    while (s_off[k + 1] <= q) ++k;
    const int j = cell_atoms[offsets[s_cell[k]] + (q - s_off[k])];
    const int s = s_shift[k];
    s4[q] = make_float4((float)((coord[3 * j] + svec[3 * s]) - ox), (float)((coord[3 * j + 1] + svec[3 * s + 1]) - oy),
                        (float)((coord[3 * j + 2] + svec[3 * s + 2]) - oz), __int_as_float(atype[j]));
    sidx[q] = s * nloc + j;
  }
  __syncthreads();
  double* wr = kr + warp * kept_cap;
  int* wi = kidx + warp * kept_cap;
  int* wt = ktype + warp * kept_cap;
  for (int a = offsets[c] + warp; a < offsets[c + 1]; a += kCellWarps) {
    const int i = cell_atoms[a];
    int* row = nlist + (size_t)i * sel.nnei;
    for (int q = lane; q < sel.nnei; q += 32) row[q] = -1;
    __syncwarp();
    if (atype[i] < 0) continue;
    const double xi = coord[3 * i], yi = coord[3 * i + 1], zi = coord[3 * i + 2];
    const int self = g.zero_shift * nloc + i;
    const float xf = (float)(xi - ox), yf = (float)(yi - oy), zf = (float)(zi - oz);
    const int r = staged_list_atom(row, wr, wi, wt, s4, sidx, total, self, xf, yf, zf, eps, coord,
                                   svec, nloc, 0, xi, yi, zi, rcut, sel, lane, status, s_tb[warp], kept_cap);
    if (r < 0 && lane == 0) fallback[c] = fallback[gridDim.x] = 1;  // more than kept_cap candidates: to the per-atom kernel
    __syncwarp();
  }
}

// C++ order (source/lib/src/fmt_nlist.cc:98-150): fp32 r^2 computed without
// contraction, (type, r^2, index) order, per-type truncation.
__global__ void __launch_bounds__(kSearchWarps * 32)
format_nlist_kernel(int* __restrict__ nlist, const double* __restrict__ coord,
                    const int* __restrict__ atype, const int* __restrict__ rows,
                    const int* __restrict__ counts, int max_nbor, int nloc, int nall, float rcut2,
                    SelInfo sel, int* __restrict__ status) {
  __shared__ float s_r[kSearchWarps][kCap];
  __shared__ int s_idx[kSearchWarps][kCap];
  __shared__ int s_type[kSearchWarps][kCap];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kSearchWarps + warp;
  if (i >= nloc) return;
  int* row = nlist + (size_t)i * sel.nnei;
  for (int q = lane; q < sel.nnei; q += 32) row[q] = -1;
  const float xi = (float)coord[3 * i], yi = (float)coord[3 * i + 1], zi = (float)coord[3 * i + 2];
  int n = 0;
  bool overflow = false;
  const int cnt = min(counts[i], max_nbor);
  for (int p0 = 0; p0 < cnt; p0 += 32) {
    const int p = p0 + lane;
    bool keep = false;
    float r2 = 0.f;
    int j = -1, tj = -1;
    if (p < cnt) {
      j = rows[(size_t)i * max_nbor + p];
      // an index outside [0, nall) is skipped rather than dereferenced
      tj = (j >= 0 && j < nall) ? atype[j] : -1;
      if (tj >= 0) {
        const float dx = __fsub_rn((float)coord[3 * j], xi);
        const float dy = __fsub_rn((float)coord[3 * j + 1], yi);
        const float dz = __fsub_rn((float)coord[3 * j + 2], zi);
        r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        keep = r2 <= rcut2;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int pos = n + __popc(m & ((1u << lane) - 1u));
    if (keep) {
      if (pos < kCap) {
        s_r[warp][pos] = r2;
        s_idx[warp][pos] = j;
        s_type[warp][pos] = tj;
      } else {
        overflow = true;
      }
    }
    n += __popc(m);
  }
  if (__any_sync(0xffffffffu, overflow)) {
    if (lane == 0) {
      atomicMax(&status[kStatusOverflow], n);
      atomicMax(&status[kStatusOverflowAtom], i + 1);
    }
    return;
  }
  __syncwarp();
  bool dropped = false;
  for (int k = lane; k < n; k += 32) {
    const float rk = s_r[warp][k];
    const int ik = s_idx[warp][k], tk = s_type[warp][k];
    int trank = 0;
    for (int m2 = 0; m2 < n; ++m2) {
      const int tm = s_type[warp][m2];
      const float rm = s_r[warp][m2];
      const int im = s_idx[warp][m2];
      trank += (tm == tk) && (rm < rk || (rm == rk && im < ik));
    }
    if (tk < sel.ntypes && trank < sel.sel[tk])
      row[sel.sec[tk] + trank] = ik;
    else
      dropped = true;
  }
  if (__any_sync(0xffffffffu, dropped) && lane == 0) atomicAdd(&status[kStatusDropped], 1);
}

// exclusive scan out[0..n] of in[0..n) (out[n] = total) by one CTA of 1024
// threads, in tiles of 4096 consecutive elements (4 per thread): coalesced
// loads, warp-shuffle scans, a running carry between tiles
__global__ void scan_kernel(int* __restrict__ out, const int* __restrict__ in, int n, const int* __restrict__ gate) {
  __shared__ int s_warp[32];
  __shared__ int s_carry;
  if (gate && !gate[0]) return;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (t == 0) s_carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 4 * blockDim.x) {
    const int idx = base + 4 * t;
    int v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = idx + k < n ? in[idx + k] : 0;
    const int local = v[0] + v[1] + v[2] + v[3];
    int x = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = s_warp[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      s_warp[lane] = w;
    }
    __syncthreads();
    int run = s_carry + (x - local) + (warp > 0 ? s_warp[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (idx + k < n) out[idx + k] = run;
      run += v[k];
    }
    __syncthreads();
    if (t == 0) s_carry += s_warp[(blockDim.x >> 5) - 1];
    __syncthreads();
  }
  if (t == 0) out[n] = s_carry;
}

// transpose: count, fill, then sort every bucket by pair id
// keys outside [0, nkeys) (padding -1 or a bad index) take no part
__global__ void tr_count_kernel(int* __restrict__ counts, const int* __restrict__ keys, long long npair,
                                int nkeys) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int k = keys[p];
  if (k < 0 || k >= nkeys) return;
  atomicAdd(&counts[k], 1);
}
__global__ void tr_fill_kernel(int* __restrict__ pairs, int* __restrict__ cursor,
                               const int* __restrict__ offsets, const int* __restrict__ keys,
                               long long npair, int nkeys) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int k = keys[p];
  if (k < 0 || k >= nkeys) return;
  pairs[offsets[k] + atomicAdd(&cursor[k], 1)] = (int)p;
}
constexpr int kTrCap = 2048;
__global__ void tr_sort_kernel(int* __restrict__ pairs, const int* __restrict__ offsets, int nkeys,
                               int* __restrict__ status) {
  __shared__ int s_v[kTrCap];
  const int k = blockIdx.x;
  if (k >= nkeys) return;
  const int beg = offsets[k], n = offsets[k + 1] - beg;
  if (n <= 1) return;
  if (n > kTrCap) {
    if (threadIdx.x == 0) {
      atomicMax(&status[kStatusOverflow], n);
      atomicMax(&status[kStatusOverflowAtom], k + 1);
    }
    return;
  }
  for (int q = threadIdx.x; q < n; q += blockDim.x) s_v[q] = pairs[beg + q];
  __syncthreads();
  int mine[kTrCap / 128];
  int cnt = 0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int v = s_v[q];
    int rank = 0;
    for (int m = 0; m < n; ++m) rank += s_v[m] < v;
    mine[cnt++] = rank;
  }
  __syncthreads();
  cnt = 0;
  for (int q = threadIdx.x; q < n; q += blockDim.x) {
    const int v = s_v[q];
    pairs[beg + mine[cnt++]] = v;
  }
}

// An external neighbour list with explicit ghost atoms (CSR: row i holds
// idx[off[i] .. off[i+1]) indices into coord_ext), formatted to typed
// sections as forward_lower does (deepmd/pt/model/model/make_model.py:
// 592-658 + nlist_distinguish_types): entries beyond rcut dropped; when
// `sorted`, ordered by (FP64 distance, index) and cut to the nearest sum(sel),
// otherwise kept in the caller's order; then per type the first sel[t].
__global__ void __launch_bounds__(kSearchWarps * 32)
format_ext_kernel(int* __restrict__ nlist, const double* __restrict__ coord, const int* __restrict__ atype,
                  const int* __restrict__ off, const int* __restrict__ idx, int nloc, int nall, double rcut,
                  SelInfo sel, int sorted, int* __restrict__ status) {
  __shared__ double s_r[kSearchWarps][kCap];
  __shared__ int s_idx[kSearchWarps][kCap];
  __shared__ int s_type[kSearchWarps][kCap];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kSearchWarps + warp;
  if (i >= nloc) return;
  int* row = nlist + (size_t)i * sel.nnei;
  for (int q = lane; q < sel.nnei; q += 32) row[q] = -1;
  if (atype[i] < 0) return;
  const double xi = coord[3 * i], yi = coord[3 * i + 1], zi = coord[3 * i + 2];
  const int beg = off[i], end = off[i + 1];
  int n = 0;
  bool overflow = false;
  for (int p0 = beg; p0 < end; p0 += 32) {
    const int p = p0 + lane;
    bool keep = false;
    double r = 0.0;
    int j = -1, tj = -1;
    if (p < end) {
      j = idx[p];
      if (j >= 0 && j < nall && (tj = atype[j]) >= 0) {
        r = dist_fma(coord[3 * j] - xi, coord[3 * j + 1] - yi, coord[3 * j + 2] - zi);
        keep = r <= rcut;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int pos = n + __popc(m & ((1u << lane) - 1u));
    if (keep) {
      if (pos < kCap) {
        s_r[warp][pos] = r;
        s_idx[warp][pos] = j;
        s_type[warp][pos] = tj;
      } else {
        overflow = true;
      }
    }
    n += __popc(m);
  }
  overflow = __any_sync(0xffffffffu, overflow);
  if (overflow) {
    if (lane == 0) {
      atomicMax(&status[kStatusOverflow], n);
      atomicMax(&status[kStatusOverflowAtom], i + 1);
    }
    return;
  }
  __syncwarp();
  for (int k = lane; k < n; k += 32) {
    const double rk = s_r[warp][k];
    const int ik = s_idx[warp][k], tk = s_type[warp][k];
    int rank = 0, trank = 0;
    for (int m2 = 0; m2 < n; ++m2) {
      // sorted: by (distance, index); caller's order: by position in the row
      const bool lt = sorted ? cand_less(s_r[warp][m2], s_idx[warp][m2], rk, ik) : m2 < k;
      rank += lt;
      trank += lt && s_type[warp][m2] == tk;
    }
    if (rank < sel.nnei && tk < sel.ntypes && trank < sel.sel[tk]) row[sel.sec[tk] + trank] = ik;
  }
}

// ---- many frames in one launch (FrameTab) ---------------------------------

__global__ void normalize_batch_kernel(double* __restrict__ out, int* __restrict__ cell_of, int* __restrict__ counts,
                                       const double* __restrict__ in, int natoms, FrameTab ft,
                                       int* __restrict__ status) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= natoms) return;
  flag_nonfinite(in + 3 * a, a, status);
  const int fr = frame_of(ft.atom_off, ft.nframes, a);
  const CellGeom& g = ft.geom[fr];
  const double x = in[3 * a], y = in[3 * a + 1], z = in[3 * a + 2];
  double fv[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    double v = fma(z, g.rec[6 + k], fma(y, g.rec[3 + k], x * g.rec[k]));
    v = v - floor(v);
    fv[k] = v;
  }
  double w[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    w[k] = fma(fv[2], g.cell[6 + k], fma(fv[1], g.cell[3 + k], fv[0] * g.cell[k]));
    out[3 * a + k] = w[k];
  }
  // cell of the wrapped position (the arithmetic of cell_count_kernel)
  int c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const double f = (w[0] * g.rec[k] + w[1] * g.rec[3 + k] + w[2] * g.rec[6 + k]) * g.ncell[k];
    int ci = (int)floor(f);
    ci = ci < 0 ? 0 : (ci >= g.ncell[k] ? g.ncell[k] - 1 : ci);
    c[k] = ci;
  }
  const int id = ft.cell_off[fr] + (c[0] * g.ncell[1] + c[1]) * g.ncell[2] + c[2];
  cell_of[a] = id;
  atomicAdd(&counts[id], 1);
}

constexpr int kBatchStageCap = 4096;

constexpr int kBatchKeptCap = 384;

size_t batch_stage_smem() {
  return (size_t)kBatchStageCap * (3 * sizeof(float) + 2 * sizeof(int)) +
         (size_t)kBatchWarps * kBatchKeptCap * (sizeof(double) + 2 * sizeof(int));
}

// nlist_cell_kernel over the cells of all frames; a cell whose stencil holds
// more than kBatchStageCap atoms, or an atom with more than kBatchKeptCap
// neighbours, is reported as an overflow
__global__ void __launch_bounds__(kBatchWarps * 32)
nlist_cell_batch_kernel(int* __restrict__ nlist, const double* __restrict__ coord, const int* __restrict__ atype,
                        const int* __restrict__ offsets, const int* __restrict__ cell_atoms,
                        const int* __restrict__ shift_pos_all, const double* __restrict__ svec_all, FrameTab ft,
                        double rcut, SelInfo sel, int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* kr = reinterpret_cast<double*>(smem);
  float4* s4 = reinterpret_cast<float4*>(kr + kBatchWarps * kBatchKeptCap);  // staged x, y, z, type bits
  int* sidx = reinterpret_cast<int*>(s4 + kBatchStageCap);
  int* kidx = sidx + kBatchStageCap;
  int* ktype = kidx + kBatchWarps * kBatchKeptCap;
  // stencil of (2 reach + 1)^3 cells, reach <= 2 per direction (a frame
  // thinner than rcut across a face has one cell and reach 2 there)
  __shared__ int s_cell[125], s_shift[125], s_off[126];
  __shared__ int s_tb[kBatchWarps][DPGB_MAX_TYPES];
  __shared__ double s_oc[3];
  const int cg = blockIdx.x, tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int fr = frame_of(ft.cell_off, ft.nframes, cg);
  const CellGeom& g = ft.geom[fr];
  const int c = cg - ft.cell_off[fr];
  const int a_beg = ft.atom_off[fr], nloc = ft.atom_off[fr + 1] - a_beg;
  const int* shift_pos = shift_pos_all + ft.spos_off[fr];
  const double* svec = svec_all + 3 * (size_t)ft.svec_off[fr];
  const int cz = c % g.ncell[2], cy = (c / g.ncell[2]) % g.ncell[1], cx = c / (g.ncell[1] * g.ncell[2]);
  const int sy_ = 2 * g.nbuff[1] + 1, sz_ = 2 * g.nbuff[2] + 1;
  const int wx = 2 * g.reach[0] + 1, wy = 2 * g.reach[1] + 1, wz = 2 * g.reach[2] + 1;
  const int nst = wx * wy * wz;
  for (int t = tid; t < nst; t += blockDim.x) {
    const int ox = t / (wy * wz) - g.reach[0], oy = (t / wz) % wy - g.reach[1], oz = t % wz - g.reach[2];
    int xw, tx, yw, ty, zw, tz;
    bool ok = wrap_cell(cx + ox, g.ncell[0], g.periodic, xw, tx) && wrap_cell(cy + oy, g.ncell[1], g.periodic, yw, ty) &&
              wrap_cell(cz + oz, g.ncell[2], g.periodic, zw, tz);
    ok = ok && abs(tx) <= g.nbuff[0] && abs(ty) <= g.nbuff[1] && abs(tz) <= g.nbuff[2];
    s_cell[t] = ok ? ft.cell_off[fr] + (xw * g.ncell[1] + yw) * g.ncell[2] + zw : -1;
    s_shift[t] = ok ? shift_pos[((tx + g.nbuff[0]) * sy_ + (ty + g.nbuff[1])) * sz_ + (tz + g.nbuff[2])] : 0;
  }
  __syncthreads();
  if (tid == 0) {
    s_off[0] = 0;
    for (int k = 0; k < nst; ++k)
      s_off[k + 1] = s_off[k] + (s_cell[k] >= 0 ? offsets[s_cell[k] + 1] - offsets[s_cell[k]] : 0);
  }
  __syncthreads();
  const int total = s_off[nst];
  if (offsets[cg] == offsets[cg + 1]) return;  // no centre atom in this cell
  if (total > kBatchStageCap) {
    if (tid == 0) {
      atomicMax(&status[kStatusOverflow], total);
      atomicMax(&status[kStatusOverflowAtom], cell_atoms[offsets[cg]] + 1);
    }
    return;
  }
  if (tid == 0) cell_centre(g, cx, cy, cz, s_oc);
  __syncthreads();
  const double ox = s_oc[0], oy = s_oc[1], oz = s_oc[2];
  const float eps = g.eps;
  for (int q = tid; q < total; q += blockDim.x) {
    int lo = 0, hi = nst;  // s_off[lo] <= q < s_off[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (s_off[mid] <= q) lo = mid; else hi = mid;
    }
    const int k = lo;
    const int j = cell_atoms[offsets[s_cell[k]] + (q - s_off[k])];  // global atom
    const int s = s_shift[k];
    s4[q] = make_float4((float)((coord[3 * j] + svec[3 * s]) - ox), (float)((coord[3 * j + 1] + svec[3 * s + 1]) - oy),
                        (float)((coord[3 * j + 2] + svec[3 * s + 2]) - oz), __int_as_float(atype[j]));
    sidx[q] = s * nloc + (j - a_beg);
  }
  __syncthreads();
  double* wr = kr + warp * kBatchKeptCap;
  int* wi = kidx + warp * kBatchKeptCap;
  int* wt = ktype + warp * kBatchKeptCap;
  for (int a = offsets[cg] + warp; a < offsets[cg + 1]; a += kBatchWarps) {
    const int i = cell_atoms[a];  // global atom
    int* row = nlist + (size_t)i * sel.nnei;
    for (int q = lane; q < sel.nnei; q += 32) row[q] = -1;
    __syncwarp();
    if (atype[i] < 0) continue;
    const double xi = coord[3 * i], yi = coord[3 * i + 1], zi = coord[3 * i + 2];
    const int self = g.zero_shift * nloc + (i - a_beg);
    const float xf = (float)(xi - ox), yf = (float)(yi - oy), zf = (float)(zi - oz);
    const int r = staged_list_atom(row, wr, wi, wt, s4, sidx, total, self, xf, yf, zf, eps, coord,
                                   svec, nloc, a_beg, xi, yi, zi, rcut, sel, lane, status, s_tb[warp], kBatchKeptCap);
    if (r < 0 && lane == 0) {
      atomicMax(&status[kStatusOverflow], -r - 1);
      atomicMax(&status[kStatusOverflowAtom], i + 1);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Skin lists: the list of an MD step reused over the next ones, as a Verlet
// list with a skin (LAMMPS neigh_modify every / check; the `ago` argument of
// DeepPot::compute, source/api_cc/src/DeepPotPT.cc:170-243).  Candidates of
// everything within rcut + skin are built on wrapped coordinates; until the
// next build the coordinates are not re-wrapped (the build's wrap offsets are
// kept), so every candidate's image shift stays the right one, and each
// evaluation selects its list at rcut from the candidates.

// gate[0] = 1 when no list exists yet, the list is `every` evaluations old,
// or an atom has moved more than skin / 2 since the build (beyond that a pair
// within rcut may be missing from the candidates)
__global__ void skin_check_kernel(int* __restrict__ gate, const double* __restrict__ coord,
                                  const double* __restrict__ ref, int n, double half2, int every) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && (gate[1] < 0 || gate[1] >= every)) gate[0] = 1;
  if (i >= n) return;
  const double dx = coord[3 * i] - ref[3 * i], dy = coord[3 * i + 1] - ref[3 * i + 1],
               dz = coord[3 * i + 2] - ref[3 * i + 2];
  if (!(dx * dx + dy * dy + dz * dz <= half2)) gate[0] = 1;
}

// build evaluation: wrap, keep the wrap offset and the reference position;
// reuse evaluation: the caller's coordinates plus the build's wrap offset
__global__ void skin_coords_kernel(double* __restrict__ out, float4* __restrict__ outf, float4* __restrict__ outflo,
                                   double* __restrict__ off, double* __restrict__ ref, const double* __restrict__ in,
                                   int n, CellGeom g, const int* __restrict__ gate, int* __restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flag_nonfinite(in + 3 * i, i, status);
  double o[3];
  if (gate[0]) {
    wrap_point(in + 3 * i, g, o);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      off[3 * i + k] = o[k] - in[3 * i + k];
      ref[3 * i + k] = in[3 * i + k];
    }
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) o[k] = in[3 * i + k] + off[3 * i + k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) out[3 * i + k] = o[k];
  const float h[3] = {(float)o[0], (float)o[1], (float)o[2]};
  outf[i] = make_float4(h[0], h[1], h[2], 0.f);
  outflo[i] = make_float4((float)(o[0] - (double)h[0]), (float)(o[1] - (double)h[1]), (float)(o[2] - (double)h[2]), 0.f);
}

// One warp per centre atom: FP32 prefilter over the candidate row (absolute
// FP32 coordinates; the margin covers their rounding), then for the packed
// survivors the displacement (r_j + shift) - r_i from the hi + lo FP32
// splits of coordinates and shifts (the exact displacement rounded once to
// FP32, as the FP64 difference rounded to FP32 would be within its bound,
// without the narrow FP64 pipe) and an FP32 distance within eps of the
// exact one.  Those decide the cutoff and the
// order unless a distance lies within eps of rcut or two within 2 eps of
// each other: then the atom is redone with exact FP64 distances.  The list
// is that of a fresh build on the same coordinates.
constexpr int kSkinWarps = 4;

// kept_cap: the per-warp kept-pair capacity of the dynamic shared memory
// (the candidate width rounded up to 32, at least 128, at most kKeptCap:
// the kept pairs cannot outnumber the candidates), so that more warps fit
// on an SM when the candidate rows are narrow
__global__ void __launch_bounds__(kSkinWarps * 32, 8)
skin_select_kernel(int* __restrict__ nlist, const int* __restrict__ cand, int ncand, int kept_cap,
                   const double* __restrict__ coord,
                   const float4* __restrict__ coordf, const float4* __restrict__ coordflo,
                   const int* __restrict__ atype, const double* __restrict__ svec, const float4* __restrict__ svecf,
                   const float4* __restrict__ svecflo, int nloc, FastDiv by_nloc, double rcut, float rcf2, float eps,
                   SelInfo sel, int* __restrict__ status) {
  extern __shared__ double s_kept[];  // [warp][kept_cap] distances, then indices, then types
  __shared__ int s_tb[kSkinWarps][DPGB_MAX_TYPES];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kSkinWarps + warp;
  if (i >= nloc) return;
  int* row = nlist + (size_t)i * sel.nnei;
  for (int q = lane; q < sel.nnei; q += 32) row[q] = -1;
  __syncwarp();
  if (atype[i] < 0) return;
  const double xi = coord[3 * i], yi = coord[3 * i + 1], zi = coord[3 * i + 2];
  const float4 fi = coordf[i], fil = coordflo[i];
  const int* c = cand + (size_t)i * ncand;
  double* wr = s_kept + (size_t)warp * kept_cap;
  float* wf = reinterpret_cast<float*>(wr);
  int* wi = reinterpret_cast<int*>(s_kept + (size_t)kSkinWarps * kept_cap) + (size_t)warp * kept_cap;
  int* wt = wi + (size_t)kSkinWarps * kept_cap;
  const unsigned below = (1u << lane) - 1u;
  int nc = 0;
#pragma unroll 2
  for (int p0 = 0; p0 < ncand; p0 += 32) {
    const int p = p0 + lane;
    const int e = p < ncand ? c[p] : -1;
    if (__all_sync(0xffffffffu, e < 0)) break;  // candidate rows are packed: padding from here on
    bool keep = false;
    if (e >= 0) {
      const int s = by_nloc.div(e), j = e - s * nloc;
      const float4 fj = coordf[j], sv = svecf[s];
      const float fx = (fj.x + sv.x) - fi.x, fy = (fj.y + sv.y) - fi.y, fz = (fj.z + sv.z) - fi.z;
      keep = fx * fx + fy * fy + fz * fz <= rcf2;
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    const int pos = nc + __popc(m & below);
    if (keep && pos < kept_cap) wi[pos] = e;
    nc += __popc(m);
  }
  if (nc > kept_cap) {
    if (lane == 0) {
      atomicMax(&status[kStatusOverflow], nc);
      atomicMax(&status[kStatusOverflowAtom], i + 1);
    }
    return;
  }
  __syncwarp();
  const float rin = (float)rcut - eps, rout = (float)rcut + eps;
  int n = 0;
  bool band = false;
#pragma unroll 2
  for (int k0 = 0; k0 < nc; k0 += 32) {
    const int k = k0 + lane;
    bool keep = false;
    float r = 0.f;
    int e = 0, t = 0;
    if (k < nc) {
      e = wi[k];
      const int s = by_nloc.div(e), j = e - s * nloc;
      t = atype[j];
      const float4 jh = coordf[j], jl = coordflo[j], sh = svecf[s], sl = svecflo[s];
      const float fx = disp_split(jh.x, jl.x, sh.x, sl.x, fi.x, fil.x);
      const float fy = disp_split(jh.y, jl.y, sh.y, sl.y, fi.y, fil.y);
      const float fz = disp_split(jh.z, jl.z, sh.z, sl.z, fi.z, fil.z);
      r = sqrtf(fx * fx + fy * fy + fz * fz);
      keep = r <= rout;
      band |= keep && r > rin;
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    __syncwarp();  // every lane has read its slot before any is overwritten
    const int pos = n + __popc(m & below);
    if (keep) {
      wf[pos] = r;
      wi[pos] = e;
      wt[pos] = t;
    }
    n += __popc(m);
  }
  band = __any_sync(0xffffffffu, band);
  __syncwarp();
  if (!band) {
    if (n <= 128) {
      sort_place_f32(row, wr, wi, wt, n, 2.f * eps, ExactDist{coord, svec, nloc, 0, xi, yi, zi}, sel, lane, status,
                     s_tb[warp]);
      return;
    }
    if (!rank_place_f32(row, wf, wi, wt, n, 2.f * eps, sel, lane, status)) return;
  }
  if (lane == 0) atomicAdd(&status[kStatusExact], 1);
  __syncwarp();
  for (int q = lane; q < sel.nnei; q += 32) row[q] = -1;
  __syncwarp();
  const int n2 = exact_keep(wr, wi, wt, n, coord, svec, nloc, 0, xi, yi, zi, rcut, lane);
  staged_rank_place(row, wr, wi, wt, n2, sel, lane, status);
}

__global__ void skin_advance_kernel(int* __restrict__ gate) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    gate[1] = gate[0] ? 1 : gate[1] + 1;
    gate[0] = 0;
  }
}

}  // namespace

size_t nlist_batch_workspace(int natoms, int ncells) {
  return sizeof(int) * (2 * (size_t)natoms + 3 * ((size_t)ncells + 1)) + 256 * 4;
}

int launch_nlist_batch(int* nlist, double* coord_out, const double* coord_in, const int* atype, int natoms,
                       int ncells, const FrameTab& ft, const double* svec, const int* shift_pos, double rcut,
                       const SelInfo& sel, void* workspace, int* status, cudaStream_t st) {
  if (natoms <= 0) return DPGB_OK;
  int* cell_of = reinterpret_cast<int*>(workspace);
  int* cell_atoms = cell_of + natoms;
  int* counts = cell_atoms + natoms;
  int* offsets = counts + (ncells + 1);
  int* cursor = offsets + (ncells + 1);
  DPGB_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (ncells + 1), st));
  DPGB_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * (ncells + 1), st));
  normalize_batch_kernel<<<ceil_div(natoms, 256), 256, 0, st>>>(coord_out, cell_of, counts, coord_in, natoms, ft,
                                                                 status);
  DPGB_TRY(check_launch("normalize_batch"));
  scan_kernel<<<1, 1024, 0, st>>>(offsets, counts, ncells, nullptr);
  DPGB_TRY(check_launch("cell_scan_batch"));
  cell_fill_kernel<<<ceil_div(natoms, 256), 256, 0, st>>>(cell_atoms, cursor, offsets, cell_of, natoms, nullptr);
  DPGB_TRY(check_launch("cell_fill_batch"));
  const size_t smem = batch_stage_smem();
  DPGB_CUDA(cudaFuncSetAttribute(nlist_cell_batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  nlist_cell_batch_kernel<<<ncells, kBatchWarps * 32, smem, st>>>(nlist, coord_out, atype, offsets, cell_atoms,
                                                                  shift_pos, svec, ft, rcut, sel, status);
  return check_launch("nlist_cell_batch");
}

int launch_format_ext(int* nlist, const double* coord_ext, const int* atype_ext, const int* off, const int* idx,
                      int nloc, int nall, double rcut, const SelInfo& sel, int sorted, int* status,
                      cudaStream_t st) {
  if (nloc <= 0) return DPGB_OK;
  format_ext_kernel<<<ceil_div(nloc, kSearchWarps), kSearchWarps * 32, 0, st>>>(nlist, coord_ext, atype_ext, off, idx,
                                                                                 nloc, nall, rcut, sel, sorted, status);
  return check_launch("format_ext");
}

int launch_normalize(double* out, const double* in, int n, const CellGeom& g, cudaStream_t st, int* status) {
  if (n <= 0) return DPGB_OK;
  normalize_kernel<<<ceil_div(n, 256), 256, 0, st>>>(out, in, n, g, status);
  return check_launch("normalize_coord");
}

int launch_skin_check(int* gate, const double* coord, const double* ref, int n, double skin, int every,
                      cudaStream_t st) {
  const double half = 0.5 * skin;
  skin_check_kernel<<<ceil_div(std::max(n, 1), 256), 256, 0, st>>>(gate, coord, ref, n, half * half, every);
  return check_launch("skin_check");
}

int launch_skin_coords(double* out, float4* outf, float4* outflo, double* off, double* ref, const double* in, int n,
                       const CellGeom& g, const int* gate, cudaStream_t st, int* status) {
  if (n <= 0) return DPGB_OK;
  skin_coords_kernel<<<ceil_div(n, 256), 256, 0, st>>>(out, outf, outflo, off, ref, in, n, g, gate, status);
  return check_launch("skin_coords");
}

int launch_skin_select(int* nlist, const int* cand, int ncand, const double* coord, const float4* coordf,
                       const float4* coordflo, const int* atype, const double* svec, const float4* svecf,
                       const float4* svecflo, int nloc, double rcut, double margin, const SelInfo& sel, int* status,
                       cudaStream_t st) {
  if (nloc <= 0) return DPGB_OK;
  const float rcf = (float)(rcut + margin);
  // displacement: the exact one rounded to FP32 (<= 2^-24 r, plus ~2^-48 of
  // the coordinates' magnitude), FP32 norm (<= 2^-22 r), x1.5
  const float eps = (float)(rcut * 1.5 * (0x1p-24 + 0x1p-22) + 1e-7);
  const int kept_cap = std::max(128, std::min(kKeptCap, (ncand + 31) / 32 * 32));
  const size_t smem = (size_t)kSkinWarps * kept_cap * (sizeof(double) + 2 * sizeof(int));  // <= 32 KB
  skin_select_kernel<<<ceil_div(nloc, kSkinWarps), kSkinWarps * 32, smem, st>>>(
      nlist, cand, ncand, kept_cap, coord, coordf, coordflo, atype, svec, svecf, svecflo, nloc, FastDiv(nloc), rcut,
      rcf * rcf, eps, sel, status);
  return check_launch("skin_select");
}

int launch_skin_advance(int* gate, cudaStream_t st) {
  skin_advance_kernel<<<1, 32, 0, st>>>(gate);
  return check_launch("skin_advance");
}

int launch_extend(double* cext, int* text, int* mapping, const double* coord, const int* atype,
                  int nloc, int nshift, const double* svec_dev, cudaStream_t st) {
  const long long tot = (long long)nloc * nshift;
  if (tot <= 0) return DPGB_OK;
  extend_kernel<<<ceil_div(tot, 256), 256, 0, st>>>(cext, text, mapping, coord, atype, nloc, nshift,
                                                     svec_dev);
  return check_launch("extend_coord");
}

size_t nlist_pt_workspace(int nloc, const CellGeom& g) {
  const size_t ncell = (size_t)g.ncell[0] * g.ncell[1] * g.ncell[2];
  return sizeof(int) * (2 * (size_t)nloc + 4 * (ncell + 1)) + 256 * 4;
}

int launch_nlist_pt(int* nlist, const double* coord, const int* atype, int nloc, const CellGeom& g,
                    const int* shift_pos_dev, const double* svec_dev, double rcut,
                    const SelInfo& sel, void* workspace, int* status, cudaStream_t st, const int* gate) {
  if (nloc <= 0) return DPGB_OK;
  const int ncell = g.ncell[0] * g.ncell[1] * g.ncell[2];
  int* cell_of = reinterpret_cast<int*>(workspace);
  int* cell_atoms = cell_of + nloc;
  int* counts = cell_atoms + nloc;
  int* offsets = counts + (ncell + 1);
  int* cursor = offsets + (ncell + 1);
  int* fallback = cursor + (ncell + 1);
  DPGB_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (ncell + 1), st));
  DPGB_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * 2 * (ncell + 1), st));  // cursor and fallback flags
  cell_count_kernel<<<ceil_div(nloc, 256), 256, 0, st>>>(cell_of, counts, coord, nloc, g, gate);
  DPGB_TRY(check_launch("cell_count"));
  scan_kernel<<<1, 1024, 0, st>>>(offsets, counts, ncell, gate);
  DPGB_TRY(check_launch("cell_scan"));
  cell_fill_kernel<<<ceil_div(nloc, 256), 256, 0, st>>>(cell_atoms, cursor, offsets, cell_of, nloc, gate);
  DPGB_TRY(check_launch("cell_fill"));
  // the staged kernel covers the 27-cell stencil; a wider stencil (a box
  // thinner than 2 rcut across a face) goes to the per-atom kernel whole
  const bool staged = g.reach[0] == 1 && g.reach[1] == 1 && g.reach[2] == 1;
  if (staged) {
    const int stage_cap = sel.flat ? kFlatStageCap : kTypedStageCap,
              kept_cap = sel.flat ? 0 : typed_kept_cap(g, nloc, rcut);
    const size_t smem = cell_stage_smem(stage_cap, kept_cap);
    DPGB_CUDA(cudaFuncSetAttribute(nlist_cell_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    nlist_cell_kernel<<<ncell, kCellWarps * 32, smem, st>>>(nlist, coord, atype, offsets, cell_atoms, shift_pos_dev,
                                                            svec_dev, nloc, g, rcut, sel, fallback, status, gate,
                                                            stage_cap, kept_cap);
    DPGB_TRY(check_launch("nlist_cell"));
  }
  // as a fallback (staged): a bounded grid whose warps stride over the atoms
  const int blocks = staged ? std::min(ceil_div(nloc, kSearchWarps), 4 * sm_count()) : ceil_div(nloc, kSearchWarps);
  nlist_pt_kernel<<<blocks, kSearchWarps * 32, 0, st>>>(nlist, coord, atype, cell_of, offsets, cell_atoms,
                                                        shift_pos_dev, svec_dev, nloc, g, rcut, sel,
                                                        staged ? fallback : nullptr, status, gate);
  return check_launch("nlist_pt");
}

int launch_format_nlist(int* nlist, const double* coord, const int* atype, const int* rows, int nall,
                        const int* counts, int max_nbor, int nloc, double rcut, const SelInfo& sel,
                        int* status, cudaStream_t st) {
  if (nloc <= 0) return DPGB_OK;
  const float rc = (float)rcut;
  format_nlist_kernel<<<ceil_div(nloc, kSearchWarps), kSearchWarps * 32, 0, st>>>(
      nlist, coord, atype, rows, counts, max_nbor, nloc, nall, rc * rc, sel, status);
  return check_launch("format_nlist");
}

size_t transpose_workspace(long long npair, int nkeys) {
  return sizeof(int) * (3 * ((size_t)nkeys + 1) + (size_t)npair) + 256;
}

int launch_transpose(Transpose& tr, const int* keys, long long npair, int nkeys, int mod,
                     void* workspace, int* status, cudaStream_t st) {
  int* counts = reinterpret_cast<int*>(workspace);
  tr.offsets = counts + (nkeys + 1);
  int* cursor = tr.offsets + (nkeys + 1);
  tr.pairs = cursor + (nkeys + 1);
  tr.nkeys = nkeys;
  DPGB_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (nkeys + 1), st));
  DPGB_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * (nkeys + 1), st));
  (void)mod;
  if (npair > 0) {
    tr_count_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(counts, keys, npair, nkeys);
    DPGB_TRY(check_launch("transpose_count"));
  }
  scan_kernel<<<1, 1024, 0, st>>>(tr.offsets, counts, nkeys, nullptr);
  DPGB_TRY(check_launch("transpose_scan"));
  if (npair > 0) {
    tr_fill_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(tr.pairs, cursor, tr.offsets, keys, npair,
                                                          nkeys);
    DPGB_TRY(check_launch("transpose_fill"));
    tr_sort_kernel<<<nkeys, 128, 0, st>>>(tr.pairs, tr.offsets, nkeys, status);
    DPGB_TRY(check_launch("transpose_sort"));
  }
  return DPGB_OK;
}

int read_status(int* status_dev, cudaStream_t st, int out[kStatusSlots]) {
  DPGB_CUDA(cudaMemcpyAsync(out, status_dev, sizeof(int) * kStatusSlots, cudaMemcpyDeviceToHost, st));
  DPGB_CUDA(cudaStreamSynchronize(st));
  return DPGB_OK;
}

}  // namespace dpgb

using namespace dpgb;


extern "C" {

int dpgb_normalize_coord(double* out, const double* coord, int natom, const double* box,
                         void* stream) {
  clear_error();
  if (natom < 0 || (natom > 0 && (!out || !coord)) || !box)
    return fail(DPGB_EINVAL, "normalize_coord: bad args (box is required)");
  CellGeom g;
  DPGB_TRY(box_geom(box, g));
  return launch_normalize(out, coord, natom, g, as_stream(stream));
}

int dpgb_extend_coord(double* cext, int* text, int* mapping, const double* coord, const int* atype,
                      int nloc, const double* box, const int* shift_idx, int nshift, void* stream) {
  clear_error();
  if (nloc < 0 || !box || !shift_idx || nshift <= 0) return fail(DPGB_EINVAL, "extend_coord: bad args");
  CellGeom g;
  DPGB_TRY(box_geom(box, g));
  std::vector<double> svec;
  shift_vectors(g, shift_idx, nshift, svec);
  DeviceBuffer d;
  DPGB_TRY(d.alloc(sizeof(double) * svec.size()));
  cudaStream_t st = as_stream(stream);
  DPGB_CUDA(cudaMemcpyAsync(d.ptr, svec.data(), sizeof(double) * svec.size(), cudaMemcpyHostToDevice, st));
  DPGB_TRY(launch_extend(cext, text, mapping, coord, atype, nloc, nshift, d.as<double>(), st));
  DPGB_CUDA(cudaStreamSynchronize(st));  // before the temporary is freed
  return DPGB_OK;
}

int dpgb_extend_input_and_build_nlist(double* coord_ext, int* atype_ext, int* mapping, int* nlist,
                                      const double* coord, const int* atype, int nframes, int nloc,
                                      const double* box, const int* shift_idx, int nshift, double rcut,
                                      const int* sel_host, int ntypes, void* stream) {
  clear_error();
  SelInfo sel;
  DPGB_TRY(sel_from_host(sel_host, ntypes, sel));
  if (nframes < 1 || nloc < 1 || !coord_ext || !atype_ext || !mapping || !nlist || !coord || !atype || !box ||
      !shift_idx || nshift < 1 || !(rcut > 0))
    return fail(DPGB_EINVAL, "extend_input_and_build_nlist: bad args");
  if ((long long)nframes * nloc * nshift >= (1LL << 31) || (long long)nframes * nloc * sel.nnei >= (1LL << 31))
    return fail(DPGB_EINVAL, "extend_input_and_build_nlist: too large");
  cudaStream_t st = as_stream(stream);
  // host geometry of every frame, then one workspace for the largest
  std::vector<CellGeom> geo(nframes);
  std::vector<std::vector<int>> spos(nframes);
  std::vector<std::vector<double>> svec(nframes);
  size_t wbytes = 0, nspos = 1;
  for (int f = 0; f < nframes; ++f) {
    for (int k = 0; k < 9; ++k)
      if (!std::isfinite(box[9 * (size_t)f + k])) return fail(DPGB_EINVAL, "extend_input_and_build_nlist: non-finite cell");
    DPGB_TRY(periodic_geom(box + 9 * (size_t)f, rcut, nshift, shift_idx, geo[f], spos[f]));
    shift_vectors(geo[f], shift_idx, nshift, svec[f]);
    wbytes = std::max(wbytes, nlist_pt_workspace(nloc, geo[f]));
    nspos = std::max(nspos, spos[f].size());
  }
  const size_t a16 = 16;
  auto up = [&](size_t b) { return (b + a16 - 1) / a16 * a16; };
  const size_t b_status = up(sizeof(int) * kStatusSlots), b_spos = up(sizeof(int) * nspos * nframes),
               b_sv = up(sizeof(double) * 3 * (size_t)nshift * nframes), b_wrap = up(sizeof(double) * 3 * nloc);
  DeviceBuffer& ws = thread_scratch(2);  // done with before the status read below returns
  DPGB_TRY(ws.alloc(b_status + b_spos + b_sv + b_wrap + wbytes + 64));
  char* base = ws.as<char>();
  int* status = reinterpret_cast<int*>(base);
  int* spos_d = reinterpret_cast<int*>(base + b_status);
  double* sv_d = reinterpret_cast<double*>(base + b_status + b_spos);
  double* wrapped = reinterpret_cast<double*>(base + b_status + b_spos + b_sv);
  void* work = base + b_status + b_spos + b_sv + b_wrap;
  std::vector<int> spos_all(nspos * nframes, -1);
  std::vector<double> sv_all(3 * (size_t)nshift * nframes);
  for (int f = 0; f < nframes; ++f) {
    std::copy(spos[f].begin(), spos[f].end(), spos_all.begin() + nspos * f);
    std::copy(svec[f].begin(), svec[f].end(), sv_all.begin() + 3 * (size_t)nshift * f);
  }
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  DPGB_CUDA(cudaMemcpyAsync(spos_d, spos_all.data(), sizeof(int) * spos_all.size(), cudaMemcpyHostToDevice, st));
  DPGB_CUDA(cudaMemcpyAsync(sv_d, sv_all.data(), sizeof(double) * sv_all.size(), cudaMemcpyHostToDevice, st));
  const size_t nall = (size_t)nloc * nshift;
  for (int f = 0; f < nframes; ++f) {  // frames in stream order share the wrap buffer and the workspace
    const double* sv_f = sv_d + 3 * (size_t)nshift * f;
    DPGB_TRY(launch_normalize(wrapped, coord + 3 * (size_t)nloc * f, nloc, geo[f], st, status));
    DPGB_TRY(launch_extend(coord_ext + 3 * nall * f, atype_ext + nall * f, mapping + nall * f, wrapped,
                           atype + (size_t)nloc * f, nloc, nshift, sv_f, st));
    DPGB_TRY(launch_nlist_pt(nlist + (size_t)nloc * sel.nnei * f, wrapped, atype + (size_t)nloc * f, nloc, geo[f],
                             spos_d + nspos * f, sv_f, rcut, sel, work, status, st));
  }
  int h[kStatusSlots];
  DPGB_TRY(read_status(status, st, h));  // also keeps the workspace alive until the kernels are done
  if (h[kStatusNonFinite] > 0) return fail(DPGB_EINVAL, "extend_input_and_build_nlist: non-finite coordinate");
  if (h[kStatusOverflow] > 0)
    return fail(DPGB_EOVERFLOW, "extend_input_and_build_nlist: atom " + std::to_string(h[kStatusOverflowAtom] - 1) +
                                    " has more than 1024 atoms within rcut");
  return DPGB_OK;
}

int dpgb_build_nlist_pt(int* nlist, const double* coord, const int* atype, int nloc,
                        const double* box, const int* shift_idx, int nshift, double rcut,
                        const int* sel_host, int ntypes, void* stream) {
  clear_error();
  SelInfo sel;
  DPGB_TRY(sel_from_host(sel_host, ntypes, sel));
  if (nloc < 0 || (nloc > 0 && (!nlist || !coord || !atype)) || !(rcut > 0))
    return fail(DPGB_EINVAL, "build_nlist_pt: bad args");
  if (nloc == 0) return DPGB_OK;
  cudaStream_t st = as_stream(stream);
  CellGeom g;
  std::vector<int> shift_pos(1, 0);
  std::vector<double> svec;
  if (box) {
    DPGB_TRY(periodic_geom(box, rcut, nshift, shift_idx, g, shift_pos));
    shift_vectors(g, shift_idx, nshift, svec);
  } else {
    // open boundary: the cell list spans the atoms' bounding box (needs the
    // coordinates on the host for the box; one copy of 24*nloc bytes)
    std::vector<double> hc((size_t)nloc * 3);
    DPGB_CUDA(cudaMemcpyAsync(hc.data(), coord, sizeof(double) * hc.size(), cudaMemcpyDeviceToHost, st));
    DPGB_CUDA(cudaStreamSynchronize(st));
    DPGB_TRY(open_geom(hc.data(), nloc, rcut, g));
    svec.assign(3, 0.0);
  }
  DeviceBuffer ws;
  const size_t wbytes = nlist_pt_workspace(nloc, g);
  const size_t extra = sizeof(int) * shift_pos.size() + sizeof(double) * svec.size() +
                       sizeof(int) * kStatusSlots + 64;
  DPGB_TRY(ws.alloc(wbytes + extra));
  char* base = ws.as<char>();
  int* status = reinterpret_cast<int*>(base);
  int* spos = status + kStatusSlots;
  double* sv = reinterpret_cast<double*>(reinterpret_cast<char*>(spos) +
                                         ((sizeof(int) * shift_pos.size() + 15) / 16) * 16);
  void* work = reinterpret_cast<char*>(sv) + ((sizeof(double) * svec.size() + 15) / 16) * 16;
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  DPGB_CUDA(cudaMemcpyAsync(spos, shift_pos.data(), sizeof(int) * shift_pos.size(), cudaMemcpyHostToDevice, st));
  DPGB_CUDA(cudaMemcpyAsync(sv, svec.data(), sizeof(double) * svec.size(), cudaMemcpyHostToDevice, st));
  DPGB_TRY(launch_nlist_pt(nlist, coord, atype, nloc, g, spos, sv, rcut, sel, work, status, st));
  int h[kStatusSlots];
  DPGB_TRY(read_status(status, st, h));
  if (h[kStatusOverflow] > 0)
    return fail(DPGB_EOVERFLOW, "build_nlist_pt: atom " + std::to_string(h[kStatusOverflowAtom] - 1) +
                                    " has more than 1024 atoms within rcut");
  return DPGB_OK;
}

int dpgb_format_nlist_a(int* nlist, const double* coord, const int* atype, const int* rows,
                        const int* counts, int max_nbor, int nloc, int nall, double rcut,
                        const int* sel_host, int ntypes, int* overflow_host, void* stream) {
  clear_error();
  SelInfo sel;
  DPGB_TRY(sel_from_host(sel_host, ntypes, sel));
  if (nloc < 0 || nall < nloc || max_nbor < 0 || (nloc > 0 && (!nlist || !coord || !atype || !counts)))
    return fail(DPGB_EINVAL, "format_nlist_a: bad args");
  if (nloc == 0) return DPGB_OK;
  cudaStream_t st = as_stream(stream);
  DeviceBuffer ws;
  DPGB_TRY(ws.alloc(sizeof(int) * kStatusSlots));
  int* status = ws.as<int>();
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  DPGB_TRY(launch_format_nlist(nlist, coord, atype, rows, nall, counts, max_nbor, nloc, rcut, sel, status, st));
  int h[kStatusSlots];
  DPGB_TRY(read_status(status, st, h));
  if (overflow_host) *overflow_host = h[kStatusDropped];
  if (h[kStatusOverflow] > 0)
    return fail(DPGB_EOVERFLOW, "format_nlist_a: row " + std::to_string(h[kStatusOverflowAtom] - 1) +
                                    " has more than 1024 candidates within rcut");
  return DPGB_OK;
}

}  // extern "C"
