// se_e2_a descriptor block on a given environment matrix, with its first and
// second derivatives: the operator form behind the deepmd.pt DescrptBlockSeA
// forward (deepmd/pt/model/descriptor/se_a.py:742-858).
//
// Per row (one local atom) and per neighbour-type section the embedding net
// G = MLP(s), s = rr[:, 0], is evaluated on the row's kept slots (the pair
// exclusion mask of deepmd/pt/utils/exclude_mask.py:104-141 removes a slot;
// padding slots are kept, as in the reference), contracted as
// xyz = sum_p rr_p^T G_p / nnei  [4, ng], and D = xyz^T xyz[:, :M]  [ng, M].
//
// All three passes share one per-pair routine: a "dual" forward through the
// MLP (values and, when asked, the tangent d/ds), and its reverse sweep, which
// returns the cotangent of s and accumulates the parameter gradients.
//   forward:          values only;
//   backward:         reverse of the values (dG -> ds, dW);
//   double backward:  reverse of values + tangents, i.e. the gradient of
//                     <a_bar, G(s)> + <a_dot_bar, G'(s)> with respect to s and
//                     the parameters (forward-over-reverse).
// Activations are recomputed in every pass, never stored between passes.
// Parameter gradients are written per (row, section) and then summed in row
// order by a second kernel: no atomics, bitwise reproducible.
#include <vector>

#include "common.cuh"

namespace dpgb {
namespace {

constexpr int kBlockThreads = 256;
constexpr int kMaxLayers = DPGB_MAX_LAYERS;
constexpr int kMaskDim = DPGB_MAX_TYPES + 1;

enum BlockMode { kModeFwd = 0, kModeBwd = 1, kModeBwdBwd = 2 };

struct BlockGeom {
  int ntypes, nnei, ng, axis, n_layer, resnet_dt, type_one_side;
  int nloc, nall, nrows;
  int sec[DPGB_MAX_TYPES + 1];
  int width[kMaxLayers + 1];  // width[0] = 1 (the input s)
  int aoff[kMaxLayers + 1];   // offset of layer l's activations in a pair's column
  int sw;                     // sum of widths (activation column length)
  int maxw;
  int woff[kMaxLayers], boff[kMaxLayers], ioff[kMaxLayers];  // per-net parameter offsets
  int pnet;                   // parameters per net
  int keep[kMaskDim * kMaskDim];
  int want_pgrad;
  int stage_w;  // the current net's parameters staged in shared memory (else read from global memory)
};

template <typename T>
__device__ __forceinline__ T tanh_b(T x);
template <>
__device__ __forceinline__ double tanh_b<double>(double x) { return tanh(x); }
template <>
__device__ __forceinline__ float tanh_b<float>(float x) { return tanhf(x); }

template <typename T>
struct Smem {
  T* w;  // the current net's parameters (staged per section)
  T *rr, *u, *X, *C, *A, *Xd;
  T *a, *ad, *t, *zd;  // [CH][sw] activations, tangents; [CH][sw] tanh, z-dot (layer l at aoff[l])
  T *bar[2], *dbar[2], *zb, *zdb;  // [CH][maxw]
  int* list;
  int* nact;
};

template <typename T>
__host__ __device__ inline size_t block_smem_elems(const BlockGeom& g, int ch) {
  size_t n = 0;
  n += 2 * (size_t)g.nnei * 4;      // rr, u
  n += 4 * (size_t)4 * g.ng;        // X, C, A, Xd
  n += 4 * (size_t)ch * g.sw;       // a, ad, t, zd
  n += 6 * (size_t)ch * g.maxw;     // bar x2, dbar x2, zb, zdb
  if (g.stage_w) n += (size_t)g.pnet;  // w
  return n;
}

template <typename T>
__device__ void carve(Smem<T>& s, const BlockGeom& g, int ch, unsigned char* base) {
  T* p = reinterpret_cast<T*>(base);
  s.w = p; p += g.stage_w ? g.pnet : 0;
  s.rr = p; p += g.nnei * 4;
  s.u = p; p += g.nnei * 4;
  s.X = p; p += 4 * g.ng;
  s.C = p; p += 4 * g.ng;
  s.A = p; p += 4 * g.ng;
  s.Xd = p; p += 4 * g.ng;
  s.a = p; p += ch * g.sw;
  s.ad = p; p += ch * g.sw;
  s.t = p; p += ch * g.sw;
  s.zd = p; p += ch * g.sw;
  s.bar[0] = p; p += ch * g.maxw;
  s.bar[1] = p; p += ch * g.maxw;
  s.dbar[0] = p; p += ch * g.maxw;
  s.dbar[1] = p; p += ch * g.maxw;
  s.zb = p; p += ch * g.maxw;
  s.zdb = p; p += ch * g.maxw;
  s.list = reinterpret_cast<int*>(p);
  s.nact = s.list + g.nnei;
}

// Dual forward of np pairs through the net at W (values, and tangents with
// a_0 = 1 when TAN).  s.a[p*sw + aoff[l] + n] = layer-l output.
template <typename T, bool TAN>
__device__ void dual_forward(const BlockGeom& g, const T* __restrict__ W, const Smem<T>& s, const int* lst, int np) {
  const int tid = threadIdx.x;
  for (int p = tid; p < np; p += blockDim.x) {
    s.a[p * g.sw] = s.rr[lst[p] * 4];
    if (TAN) s.ad[p * g.sw] = T(1);
  }
  __syncthreads();
  for (int l = 1; l <= g.n_layer; ++l) {
    const int nin = g.width[l - 1], nout = g.width[l];
    const T* Wm = W + g.woff[l - 1];
    const T* b = W + g.boff[l - 1];
    const T* id = g.resnet_dt ? W + g.ioff[l - 1] : nullptr;
    const int ai = g.aoff[l - 1], ao = g.aoff[l];
    // one thread: four outputs n = t, t + n4, t + 2 n4, t + 3 n4 of one
    // pair (x[k] read once for the four; consecutive threads read
    // consecutive weights; each output's sum in the same order as one at a
    // time)
    const int n4 = (nout + 3) >> 2;
    for (int q = tid; q < np * n4; q += blockDim.x) {
      const int p = q / n4, t0 = q - p * n4;
      const T* x = s.a + p * g.sw + ai;
      const T* xd = s.ad + p * g.sw + ai;
      T z[4], zd[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        z[j] = t0 + j * n4 < nout ? b[t0 + j * n4] : T(0);
        zd[j] = T(0);
      }
      for (int k = 0; k < nin; ++k) {
        const T xk = x[k];
        const T xdk = TAN ? xd[k] : T(0);
        const T* wr = Wm + k * nout + t0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (t0 + j * n4 < nout) {
            const T w = wr[j * n4];
            z[j] += xk * w;
            if (TAN) zd[j] += xdk * w;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int n = t0 + j * n4;
        if (n >= nout) break;
        const T t = tanh_b(z[j]);
        T y = id ? t * id[n] : t;
        if (nout == nin) y += x[n];
        else if (nout == 2 * nin) y += x[n % nin];
        s.a[p * g.sw + ao + n] = y;
        s.t[p * g.sw + ao + n] = t;
        if (TAN) {
          const T td = (T(1) - t * t) * zd[j];
          T yd = id ? td * id[n] : td;
          if (nout == nin) yd += xd[n];
          else if (nout == 2 * nin) yd += xd[n % nin];
          s.ad[p * g.sw + ao + n] = yd;
          s.zd[p * g.sw + ao + n] = zd[j];
        }
      }
    }
    __syncthreads();
  }
}

// Reverse sweep: on entry s.bar[0] (and s.dbar[0] when TAN) hold the
// cotangents of the last layer's output [np][nout_L]; on exit the returned
// buffer index holds the cotangent of s in column 0.  Parameter gradients of
// this chunk are added to pg (this row's slice for the net) when non-null.
template <typename T, bool TAN>
__device__ int dual_reverse(const BlockGeom& g, const T* __restrict__ W, const Smem<T>& s, int np,
                            T* __restrict__ pg) {
  const int tid = threadIdx.x;
  int cur = 0;
  for (int l = g.n_layer; l >= 1; --l) {
    const int nin = g.width[l - 1], nout = g.width[l];
    const T* Wm = W + g.woff[l - 1];
    const T* id = g.resnet_dt ? W + g.ioff[l - 1] : nullptr;
    const int ai = g.aoff[l - 1], ao = g.aoff[l];
    const T* yb = s.bar[cur];
    const T* ydb = s.dbar[cur];
    for (int q = tid; q < np * nout; q += blockDim.x) {
      const int p = q / nout, n = q - p * nout;
      const T t = s.t[p * g.sw + ao + n];
      const T idn = id ? id[n] : T(1);
      T tb = yb[p * g.maxw + n] * idn;
      if (TAN) {
        const T tdb = ydb[p * g.maxw + n] * idn;
        const T zd = s.zd[p * g.sw + ao + n];
        s.zdb[p * g.maxw + n] = tdb * (T(1) - t * t);
        tb += tdb * (T(-2) * t * zd);
      }
      s.zb[p * g.maxw + n] = tb * (T(1) - t * t);
    }
    __syncthreads();
    if (pg) {
      T* gW = pg + g.woff[l - 1];
      // one thread: n = t, t + n4, t + 2 n4, t + 3 n4 of one k (each sum
      // in pair order; consecutive threads on consecutive n)
      const int n4 = (nout + 3) >> 2;
      for (int q = tid; q < nin * n4; q += blockDim.x) {
        const int k = q / n4, t0 = q - k * n4;
        T acc[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = t0 + j * n4 < nout ? gW[k * nout + t0 + j * n4] : T(0);
        for (int p = 0; p < np; ++p) {
          const T av = s.a[p * g.sw + ai + k];
          const T* zr = s.zb + p * g.maxw + t0;
          const T adv = TAN ? s.ad[p * g.sw + ai + k] : T(0);
          const T* zdr = s.zdb + p * g.maxw + t0;
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            if (t0 + j * n4 < nout) {
              acc[j] += av * zr[j * n4];
              if (TAN) acc[j] += adv * zdr[j * n4];
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (t0 + j * n4 < nout) gW[k * nout + t0 + j * n4] = acc[j];
      }
      T* gb = pg + g.boff[l - 1];
      T* gi = g.resnet_dt ? pg + g.ioff[l - 1] : nullptr;
      for (int n = tid; n < nout; n += blockDim.x) {
        T ab = gb[n];
        for (int p = 0; p < np; ++p) ab += s.zb[p * g.maxw + n];
        gb[n] = ab;
        if (gi) {
          T ai2 = gi[n];
          for (int p = 0; p < np; ++p) {
            const T t = s.t[p * g.sw + ao + n];
            ai2 += yb[p * g.maxw + n] * t;
            if (TAN) ai2 += ydb[p * g.maxw + n] * ((T(1) - t * t) * s.zd[p * g.sw + ao + n]);
          }
          gi[n] = ai2;
        }
      }
    }
    T* xb = s.bar[1 - cur];
    T* xdb = s.dbar[1 - cur];
    // one thread: k = t, t + k4, t + 2 k4, t + 3 k4 of one pair (zb[n]
    // read once for the four; each sum in n order)
    const int k4 = (nin + 3) >> 2;
    for (int q = tid; q < np * k4; q += blockDim.x) {
      const int p = q / k4, t0 = q - p * k4;
      T acc[4] = {T(0), T(0), T(0), T(0)}, accd[4] = {T(0), T(0), T(0), T(0)};
      const T* zr = s.zb + p * g.maxw;
      const T* zdr = s.zdb + p * g.maxw;
      for (int n = 0; n < nout; ++n) {
        const T zn = zr[n];
        const T zdn = TAN ? zdr[n] : T(0);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int k = t0 + j * k4;
          if (k < nin) {
            const T w = Wm[k * nout + n];
            acc[j] += zn * w;
            if (TAN) accd[j] += zdn * w;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = t0 + j * k4;
        if (k >= nin) break;
        T a0 = acc[j], d0 = accd[j];
        if (nout == nin) {
          a0 += yb[p * g.maxw + k];
          if (TAN) d0 += ydb[p * g.maxw + k];
        } else if (nout == 2 * nin) {
          a0 += yb[p * g.maxw + k] + yb[p * g.maxw + k + nin];
          if (TAN) d0 += ydb[p * g.maxw + k] + ydb[p * g.maxw + k + nin];
        }
        xb[p * g.maxw + k] = a0;
        if (TAN) xdb[p * g.maxw + k] = d0;
      }
    }
    __syncthreads();
    cur = 1 - cur;
  }
  return cur;
}

// the net's parameters into shared memory (section_list's barriers order
// this against the previous section's last reads; the barrier here against
// the next reads).  (A transposed copy for the reverse sweep measured
// slower: the transposition costs more than the bank conflicts it saves.)
template <typename T>
__device__ void stage_net(const BlockGeom& g, T* __restrict__ w, const T* __restrict__ src) {
  for (int q = threadIdx.x; q < g.pnet; q += blockDim.x) w[q] = src[q];
  __syncthreads();
}

__device__ __forceinline__ int net_of(const BlockGeom& g, int sec, int ti) {
  return g.type_one_side ? sec : sec * g.ntypes + ti;
}

// kept slots of section sec of this row -> s.list, count -> *s.nact
template <typename T>
__device__ void section_list(const BlockGeom& g, const Smem<T>& s, const int* __restrict__ nlist_row,
                             const int* __restrict__ atype_f, int ti, int sec) {
  __syncthreads();
  if (threadIdx.x < 32) {  // warp 0, 32 slots at a time, in slot order
    const int lane = threadIdx.x;
    int n = 0;
    for (int k0 = g.sec[sec]; k0 < g.sec[sec + 1]; k0 += 32) {
      const int k = k0 + lane;
      bool kept = false;
      if (k < g.sec[sec + 1]) {
        const int j = nlist_row[k];
        int tj = (j >= 0 && j < g.nall) ? atype_f[j] : g.ntypes;
        if (tj < 0 || tj > g.ntypes) tj = g.ntypes;
        kept = g.keep[ti * kMaskDim + tj] != 0;
      }
      const unsigned m = __ballot_sync(0xffffffffu, kept);
      if (kept) s.list[n + __popc(m & ((1u << lane) - 1u))] = k;
      n += __popc(m);
    }
    if (lane == 0) *s.nact = n;
  }
  __syncthreads();
}

// dL/dX from dD (and a direct dX): C[c][k] = sum_m gD[k][m] X[c][m] + [k<M] sum_n gD[n][k] X[c][n] (+ gX)
template <typename T>
__device__ void dD_to_dX(const BlockGeom& g, const T* __restrict__ gD, const T* __restrict__ gX, const T* X, T* out) {
  const int M = g.axis, ng = g.ng;
  for (int q = threadIdx.x; q < 4 * ng; q += blockDim.x) {
    const int c = q / ng, k = q - c * ng;
    T acc = gX ? gX[q] : T(0);
    for (int m = 0; m < M; ++m) acc += gD[k * M + m] * X[c * ng + m];
    if (k < M)
      for (int n = 0; n < ng; ++n) acc += gD[n * M + k] * X[c * ng + n];
    out[q] = acc;
  }
}

template <typename T, int CH, int MODE>
__global__ void __launch_bounds__(kBlockThreads)
se_a_block_kernel(BlockGeom g, const T* __restrict__ params, const T* __restrict__ rr, const int* __restrict__ nlist,
                  const int* __restrict__ atype_ext, const T* __restrict__ xyz_in, const T* __restrict__ gD,
                  const T* __restrict__ gX, const T* __restrict__ u, T* __restrict__ out_D, T* __restrict__ out_X,
                  T* __restrict__ out_rr, T* __restrict__ out_gD, T* __restrict__ out_gX, T* __restrict__ pgrad) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem<T> s;
  carve(s, g, CH, smem_raw);
  const int row = blockIdx.x, tid = threadIdx.x;
  const int f = row / g.nloc, i = row - f * g.nloc;
  const int* atype_f = atype_ext + (size_t)f * g.nall;
  const int ti = atype_f[i];
  const int* nl = nlist + (size_t)row * g.nnei;
  const int ng = g.ng, M = g.axis;
  const T inv_nnei = T(1) / T(g.nnei);
  const bool pgr = MODE != kModeFwd && g.want_pgrad && pgrad;
  T* prow = pgr ? pgrad + (size_t)row * g.ntypes * g.pnet : nullptr;
  if (pgr)
    for (int q = tid; q < g.ntypes * g.pnet; q += blockDim.x) prow[q] = T(0);
  if (ti < 0 || ti >= g.ntypes) {  // rows without a type contribute nothing
    if (MODE == kModeFwd) {
      for (int q = tid; q < ng * M; q += blockDim.x) out_D[(size_t)row * ng * M + q] = T(0);
      for (int q = tid; q < 4 * ng; q += blockDim.x) out_X[(size_t)row * 4 * ng + q] = T(0);
    } else {
      for (int q = tid; q < 4 * g.nnei; q += blockDim.x) out_rr[(size_t)row * 4 * g.nnei + q] = T(0);
      if (MODE == kModeBwdBwd) {
        for (int q = tid; q < ng * M; q += blockDim.x) out_gD[(size_t)row * ng * M + q] = T(0);
        if (out_gX)
          for (int q = tid; q < 4 * ng; q += blockDim.x) out_gX[(size_t)row * 4 * ng + q] = T(0);
      }
    }
    return;
  }
  for (int q = tid; q < 4 * g.nnei; q += blockDim.x) {
    s.rr[q] = rr[(size_t)row * 4 * g.nnei + q];
    if (MODE == kModeBwdBwd) s.u[q] = u[(size_t)row * 4 * g.nnei + q];
    if (MODE != kModeFwd) out_rr[(size_t)row * 4 * g.nnei + q] = T(0);
  }
  for (int q = tid; q < 4 * ng; q += blockDim.x) {
    s.X[q] = MODE == kModeBwd ? xyz_in[(size_t)row * 4 * ng + q] : T(0);
    s.Xd[q] = T(0);
  }
  __syncthreads();

  // pass 1 (forward and double backward): X (and its tangent Xd along u)
  if (MODE != kModeBwd) {
    for (int sec = 0; sec < g.ntypes; ++sec) {
      section_list(g, s, nl, atype_f, ti, sec);
      const int nact = *s.nact;
      const T* W = params + (size_t)net_of(g, sec, ti) * g.pnet;
      if (g.stage_w) {
        stage_net(g, s.w, W);
        W = s.w;
      }
      for (int c0 = 0; c0 < nact; c0 += CH) {
        const int np = min(CH, nact - c0);
        const int* lst = s.list + c0;
        dual_forward<T, MODE == kModeBwdBwd>(g, W, s, lst, np);
        const int aL = g.aoff[g.n_layer];
        for (int q = tid; q < 4 * ng; q += blockDim.x) {
          const int c = q / ng, n = q - c * ng;
          T acc = T(0), accd = T(0);
          for (int p = 0; p < np; ++p) {
            const int k = lst[p];
            const T G = s.a[p * g.sw + aL + n];
            acc += s.rr[k * 4 + c] * G;
            if (MODE == kModeBwdBwd) accd += s.u[k * 4 + c] * G + s.u[k * 4] * s.rr[k * 4 + c] * s.ad[p * g.sw + aL + n];
          }
          s.X[q] += acc;
          if (MODE == kModeBwdBwd) s.Xd[q] += accd;
        }
        __syncthreads();
      }
    }
    for (int q = tid; q < 4 * ng; q += blockDim.x) {
      s.X[q] *= inv_nnei;
      s.Xd[q] *= inv_nnei;
    }
    __syncthreads();
  }

  if (MODE == kModeFwd) {
    for (int q = tid; q < 4 * ng; q += blockDim.x) out_X[(size_t)row * 4 * ng + q] = s.X[q];
    for (int q = tid; q < ng * M; q += blockDim.x) {
      const int n = q / M, m = q - n * M;
      T acc = T(0);
#pragma unroll
      for (int c = 0; c < 4; ++c) acc += s.X[c * ng + n] * s.X[c * ng + m];
      out_D[(size_t)row * ng * M + q] = acc;
    }
    return;
  }

  // C = dL/dX; in the double backward also A (the same map applied to Xd),
  // the cotangent of dD (Q'(X) Xd) and of the direct dX (Xd)
  const T* gDr = gD + (size_t)row * ng * M;
  const T* gXr = gX ? gX + (size_t)row * 4 * ng : nullptr;
  dD_to_dX(g, gDr, gXr, s.X, s.C);
  if (MODE == kModeBwdBwd) {
    dD_to_dX(g, gDr, (const T*)nullptr, s.Xd, s.A);
    for (int q = tid; q < ng * M; q += blockDim.x) {
      const int n = q / M, m = q - n * M;
      T acc = T(0);
#pragma unroll
      for (int c = 0; c < 4; ++c) acc += s.Xd[c * ng + n] * s.X[c * ng + m] + s.X[c * ng + n] * s.Xd[c * ng + m];
      out_gD[(size_t)row * ng * M + q] = acc;
    }
    if (out_gX)
      for (int q = tid; q < 4 * ng; q += blockDim.x) out_gX[(size_t)row * 4 * ng + q] = s.Xd[q];
  }
  __syncthreads();

  // pass 2: per pair cotangents, reverse sweep
  T* orr = out_rr + (size_t)row * 4 * g.nnei;
  const int aL = g.aoff[g.n_layer];
  for (int sec = 0; sec < g.ntypes; ++sec) {
    section_list(g, s, nl, atype_f, ti, sec);
    const int nact = *s.nact;
    const int e = net_of(g, sec, ti);
    const T* W = params + (size_t)e * g.pnet;
    if (g.stage_w) {
      stage_net(g, s.w, W);
      W = s.w;
    }
    T* pg = pgr ? prow + (size_t)sec * g.pnet : nullptr;
    for (int c0 = 0; c0 < nact; c0 += CH) {
      const int np = min(CH, nact - c0);
      const int* lst = s.list + c0;
      dual_forward<T, MODE == kModeBwdBwd>(g, W, s, lst, np);
      // cotangents of the last layer and the direct rr terms
      for (int q = tid; q < np * ng; q += blockDim.x) {
        const int p = q / ng, n = q - p * ng;
        const int k = lst[p];
        T ab = T(0), adb = T(0);
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          if (MODE == kModeBwd) {
            ab += s.C[c * ng + n] * s.rr[k * 4 + c];
          } else {
            ab += s.A[c * ng + n] * s.rr[k * 4 + c] + s.C[c * ng + n] * s.u[k * 4 + c];
            adb += s.C[c * ng + n] * s.rr[k * 4 + c];
          }
        }
        s.bar[0][p * g.maxw + n] = ab * inv_nnei;
        if (MODE == kModeBwdBwd) s.dbar[0][p * g.maxw + n] = adb * s.u[k * 4] * inv_nnei;
      }
      for (int q = tid; q < np * 4; q += blockDim.x) {
        const int p = q >> 2, c = q & 3;
        const int k = lst[p];
        T acc = T(0);
        for (int n = 0; n < ng; ++n) {
          if (MODE == kModeBwd) {
            acc += s.C[c * ng + n] * s.a[p * g.sw + aL + n];
          } else {
            acc += s.A[c * ng + n] * s.a[p * g.sw + aL + n] + s.u[k * 4] * s.C[c * ng + n] * s.ad[p * g.sw + aL + n];
          }
        }
        orr[k * 4 + c] = acc * inv_nnei;
      }
      __syncthreads();
      const int fin = dual_reverse<T, MODE == kModeBwdBwd>(g, W, s, np, pg);
      for (int p = tid; p < np; p += blockDim.x) orr[lst[p] * 4] += s.bar[fin][p * g.maxw];
      __syncthreads();
    }
  }
}

// gparams[e][k] = sum over rows r (in order) and sections s with net(r, s) == e of partial[r][s][k]
// gparams[e][k] = sum over rows r (in order) and sections s with net(r, s) == e
// of partial[r][s][k], in two levels: sums over chunks of kReduceRows rows
// (in row order), then the chunk sums in chunk order
constexpr int kReduceRows = 64;

template <typename T>
__global__ void pgrad_chunk_kernel(T* __restrict__ chunk_out, const T* __restrict__ part,
                                   const int* __restrict__ atype_ext, BlockGeom g, int nnets) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nnets * g.pnet) return;
  const int e = (int)(q / g.pnet), k = (int)(q - (long long)e * g.pnet);
  const int sec = g.type_one_side ? e : e / g.ntypes;
  const int tcen = g.type_one_side ? -1 : e % g.ntypes;
  const int r0 = blockIdx.y * kReduceRows, r1 = min(g.nrows, r0 + kReduceRows);
  T acc = T(0);
  for (int r = r0; r < r1; ++r) {
    const int f = r / g.nloc, i = r - f * g.nloc;
    const int ti = atype_ext[(size_t)f * g.nall + i];
    if (ti < 0 || ti >= g.ntypes) continue;
    if (tcen >= 0 && ti != tcen) continue;
    acc += part[((size_t)r * g.ntypes + sec) * g.pnet + k];
  }
  chunk_out[(size_t)blockIdx.y * nnets * g.pnet + q] = acc;
}

template <typename T>
__global__ void pgrad_final_kernel(T* __restrict__ out, const T* __restrict__ chunk_out, long long n, int nchunk) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  T acc = T(0);
  for (int c = 0; c < nchunk; ++c) acc += chunk_out[(size_t)c * n + q];
  out[q] = acc;
}

int make_geom(const dpgb_se_a_block* b, int nf, int nloc, int nall, BlockGeom& g) {
  if (!b) return fail(DPGB_EINVAL, "se_a_block: NULL description");
  if (b->ntypes < 1 || b->ntypes > DPGB_MAX_TYPES) return fail(DPGB_EINVAL, "se_a_block: ntypes out of range");
  if (b->n_layer < 1 || b->n_layer > kMaxLayers) return fail(DPGB_EINVAL, "se_a_block: n_layer out of range");
  if (nf < 1 || nloc < 0 || nall < nloc) return fail(DPGB_EINVAL, "se_a_block: bad sizes");
  g = BlockGeom{};
  g.ntypes = b->ntypes;
  g.sec[0] = 0;
  for (int t = 0; t < g.ntypes; ++t) {
    if (b->sel[t] < 0) return fail(DPGB_EINVAL, "se_a_block: negative sel");
    g.sec[t + 1] = g.sec[t] + b->sel[t];
  }
  g.nnei = g.sec[g.ntypes];
  if (g.nnei < 1) return fail(DPGB_EINVAL, "se_a_block: empty sel");
  g.n_layer = b->n_layer;
  g.width[0] = 1;
  g.maxw = 1;
  for (int l = 0; l < g.n_layer; ++l) {
    if (b->neuron[l] < 1 || b->neuron[l] > 1024) return fail(DPGB_EINVAL, "se_a_block: bad neuron width");
    g.width[l + 1] = b->neuron[l];
    g.maxw = std::max(g.maxw, b->neuron[l]);
  }
  g.ng = g.width[g.n_layer];
  g.axis = b->axis_neuron;
  if (g.axis < 1 || g.axis > g.ng) return fail(DPGB_EINVAL, "se_a_block: axis_neuron must be in [1, ng]");
  g.resnet_dt = b->resnet_dt ? 1 : 0;
  g.type_one_side = b->type_one_side ? 1 : 0;
  g.sw = 0;
  for (int l = 0; l <= g.n_layer; ++l) {
    g.aoff[l] = g.sw;
    g.sw += g.width[l];
  }
  int off = 0;
  for (int l = 0; l < g.n_layer; ++l) {
    g.woff[l] = off;
    off += g.width[l] * g.width[l + 1];
    g.boff[l] = off;
    off += g.width[l + 1];
    g.ioff[l] = off;
    if (g.resnet_dt) off += g.width[l + 1];
  }
  g.pnet = off;
  for (int a = 0; a < kMaskDim * kMaskDim; ++a) g.keep[a] = 1;
  for (int a = 0; a <= g.ntypes; ++a)
    for (int c = 0; c <= g.ntypes; ++c) g.keep[a * kMaskDim + c] = b->pair_keep[a * kMaskDim + c] ? 1 : 0;
  g.nloc = nloc;
  g.nall = nall;
  g.nrows = nf * nloc;
  return DPGB_OK;
}

template <typename T>
constexpr int chunk_of() {
  return sizeof(T) == 8 ? 8 : 32;  // pairs per chunk (shared-memory arrays of chunk x width)
}

template <typename T>
size_t smem_bytes(const BlockGeom& g) {
  return block_smem_elems<T>(g, chunk_of<T>()) * sizeof(T) + sizeof(int) * (g.nnei + 1) + 16;
}

template <typename T, int MODE>
int launch_block(BlockGeom g, const T* params, const T* rr, const int* nlist, const int* atype, const T* xyz_in,
                 const T* gD, const T* gX, const T* u, T* oD, T* oX, T* orr, T* ogD, T* ogX, T* pg, cudaStream_t st) {
  constexpr int CH = chunk_of<T>();
  // FP32: the staged weights take their reads off L1; FP64 is bound by its
  // narrow pipe, where two CTAs per SM without them do better
  g.stage_w = sizeof(T) == 4;
  size_t smem = smem_bytes<T>(g);
  if (smem > 227 * 1024) {  // no room for the weights: read them from global memory
    g.stage_w = 0;
    smem = smem_bytes<T>(g);
  }
  if (smem > 227 * 1024) return fail(DPGB_EINVAL, "se_a_block: widths too large for one CTA's shared memory");
  auto k = se_a_block_kernel<T, CH, MODE>;
  DPGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (g.nrows == 0) return DPGB_OK;
  k<<<g.nrows, kBlockThreads, smem, st>>>(g, params, rr, nlist, atype, xyz_in, gD, gX, u, oD, oX, orr, ogD, ogX, pg);
  return check_launch("se_a_block");
}

template <typename T>
int reduce_pgrad(const BlockGeom& g, T* gparams, T* part, const int* atype, cudaStream_t st) {
  const int nnets = g.type_one_side ? g.ntypes : g.ntypes * g.ntypes;
  const long long n = (long long)nnets * g.pnet;
  const int nchunk = ceil_div(g.nrows, kReduceRows);
  T* chunk_out = part + (size_t)g.nrows * g.ntypes * g.pnet;  // after the row partials in the workspace
  pgrad_chunk_kernel<T><<<dim3(ceil_div(n, 128), nchunk), 128, 0, st>>>(chunk_out, part, atype, g, nnets);
  DPGB_TRY(check_launch("se_a_block_pgrad_chunks"));
  pgrad_final_kernel<T><<<ceil_div(n, 128), 128, 0, st>>>(gparams, chunk_out, n, nchunk);
  return check_launch("se_a_block_pgrad_reduce");
}

template <typename T>
int block_fwd(const dpgb_se_a_block* b, const T* params, const T* rr, const int* nlist, const int* atype, int nf,
              int nloc, int nall, T* D, T* xyz, void* stream) {
  clear_error();
  BlockGeom g;
  DPGB_TRY(make_geom(b, nf, nloc, nall, g));
  if (!params || !rr || !nlist || !atype || !D || !xyz) return fail(DPGB_EINVAL, "se_a_block_fwd: NULL pointer");
  return launch_block<T, kModeFwd>(g, params, rr, nlist, atype, nullptr, nullptr, nullptr, nullptr, D, xyz, nullptr,
                                   nullptr, nullptr, nullptr, as_stream(stream));
}

template <typename T>
size_t workspace_bytes(const BlockGeom& g) {
  const size_t nnets = g.type_one_side ? g.ntypes : (size_t)g.ntypes * g.ntypes;
  return sizeof(T) * ((size_t)g.nrows * g.ntypes * g.pnet + (size_t)ceil_div(g.nrows, kReduceRows) * nnets * g.pnet);
}

template <typename T>
int block_bwd(const dpgb_se_a_block* b, const T* params, const T* rr, const int* nlist, const int* atype, int nf,
              int nloc, int nall, const T* xyz, const T* gD, const T* gX, T* grr, T* gparams, void* ws,
              size_t ws_bytes, void* stream) {
  clear_error();
  BlockGeom g;
  DPGB_TRY(make_geom(b, nf, nloc, nall, g));
  if (!params || !rr || !nlist || !atype || !xyz || !gD || !grr) return fail(DPGB_EINVAL, "se_a_block_bwd: NULL pointer");
  g.want_pgrad = gparams != nullptr;
  if (gparams && (!ws || ws_bytes < workspace_bytes<T>(g)))
    return fail(DPGB_EINVAL, "se_a_block_bwd: workspace missing or smaller than dpgb_se_a_block_workspace_bytes");
  cudaStream_t st = as_stream(stream);
  DPGB_TRY((launch_block<T, kModeBwd>(g, params, rr, nlist, atype, xyz, gD, gX, nullptr, nullptr, nullptr, grr,
                                      nullptr, nullptr, gparams ? (T*)ws : nullptr, st)));
  if (gparams && g.nrows > 0) DPGB_TRY(reduce_pgrad<T>(g, gparams, (T*)ws, atype, st));
  return DPGB_OK;
}

template <typename T>
int block_bwd_bwd(const dpgb_se_a_block* b, const T* params, const T* rr, const int* nlist, const int* atype, int nf,
                  int nloc, int nall, const T* gD, const T* gX, const T* u_rr, T* g_gD, T* g_gX, T* g_rr, T* g_params,
                  void* ws, size_t ws_bytes, void* stream) {
  clear_error();
  BlockGeom g;
  DPGB_TRY(make_geom(b, nf, nloc, nall, g));
  if (!params || !rr || !nlist || !atype || !gD || !u_rr || !g_gD || !g_rr)
    return fail(DPGB_EINVAL, "se_a_block_bwd_bwd: NULL pointer");
  g.want_pgrad = g_params != nullptr;
  if (g_params && (!ws || ws_bytes < workspace_bytes<T>(g)))
    return fail(DPGB_EINVAL, "se_a_block_bwd_bwd: workspace missing or smaller than dpgb_se_a_block_workspace_bytes");
  cudaStream_t st = as_stream(stream);
  DPGB_TRY((launch_block<T, kModeBwdBwd>(g, params, rr, nlist, atype, nullptr, gD, gX, u_rr, nullptr, nullptr, g_rr,
                                         g_gD, g_gX, g_params ? (T*)ws : nullptr, st)));
  if (g_params && g.nrows > 0) DPGB_TRY(reduce_pgrad<T>(g, g_params, (T*)ws, atype, st));
  return DPGB_OK;
}

}  // namespace
}  // namespace dpgb

using namespace dpgb;

extern "C" {

long long dpgb_se_a_block_param_count(const dpgb_se_a_block* b) {
  BlockGeom g;
  if (make_geom(b, 1, 0, 0, g) != DPGB_OK) return -1;
  return (long long)g.pnet * (g.type_one_side ? g.ntypes : g.ntypes * g.ntypes);
}

size_t dpgb_se_a_block_workspace_bytes(const dpgb_se_a_block* b, int nf, int nloc, int precision_bytes) {
  BlockGeom g;
  if (make_geom(b, nf, nloc, nloc, g) != DPGB_OK) return 0;
  return precision_bytes == 8 ? workspace_bytes<double>(g) : workspace_bytes<float>(g);
}

int dpgb_se_a_block_fwd_f64(const dpgb_se_a_block* b, const double* params, const double* rr, const int* nlist,
                            const int* atype_ext, int nf, int nloc, int nall, double* descriptor, double* xyz,
                            void* stream) {
  return block_fwd<double>(b, params, rr, nlist, atype_ext, nf, nloc, nall, descriptor, xyz, stream);
}
int dpgb_se_a_block_fwd_f32(const dpgb_se_a_block* b, const float* params, const float* rr, const int* nlist,
                            const int* atype_ext, int nf, int nloc, int nall, float* descriptor, float* xyz,
                            void* stream) {
  return block_fwd<float>(b, params, rr, nlist, atype_ext, nf, nloc, nall, descriptor, xyz, stream);
}

int dpgb_se_a_block_bwd_f64(const dpgb_se_a_block* b, const double* params, const double* rr, const int* nlist,
                            const int* atype_ext, int nf, int nloc, int nall, const double* xyz,
                            const double* g_descriptor, const double* g_xyz, double* g_rr, double* g_params,
                            void* workspace, size_t workspace_bytes, void* stream) {
  return block_bwd<double>(b, params, rr, nlist, atype_ext, nf, nloc, nall, xyz, g_descriptor, g_xyz, g_rr, g_params,
                           workspace, workspace_bytes, stream);
}
int dpgb_se_a_block_bwd_f32(const dpgb_se_a_block* b, const float* params, const float* rr, const int* nlist,
                            const int* atype_ext, int nf, int nloc, int nall, const float* xyz,
                            const float* g_descriptor, const float* g_xyz, float* g_rr, float* g_params,
                            void* workspace, size_t workspace_bytes, void* stream) {
  return block_bwd<float>(b, params, rr, nlist, atype_ext, nf, nloc, nall, xyz, g_descriptor, g_xyz, g_rr, g_params,
                          workspace, workspace_bytes, stream);
}

int dpgb_se_a_block_bwd_bwd_f64(const dpgb_se_a_block* b, const double* params, const double* rr, const int* nlist,
                                const int* atype_ext, int nf, int nloc, int nall, const double* g_descriptor,
                                const double* g_xyz, const double* u_rr, double* gg_descriptor, double* gg_xyz,
                                double* gg_rr, double* gg_params, void* workspace, size_t workspace_bytes,
                                void* stream) {
  return block_bwd_bwd<double>(b, params, rr, nlist, atype_ext, nf, nloc, nall, g_descriptor, g_xyz, u_rr,
                               gg_descriptor, gg_xyz, gg_rr, gg_params, workspace, workspace_bytes, stream);
}
int dpgb_se_a_block_bwd_bwd_f32(const dpgb_se_a_block* b, const float* params, const float* rr, const int* nlist,
                                const int* atype_ext, int nf, int nloc, int nall, const float* g_descriptor,
                                const float* g_xyz, const float* u_rr, float* gg_descriptor, float* gg_xyz,
                                float* gg_rr, float* gg_params, void* workspace, size_t workspace_bytes,
                                void* stream) {
  return block_bwd_bwd<float>(b, params, rr, nlist, atype_ext, nf, nloc, nall, g_descriptor, g_xyz, u_rr,
                              gg_descriptor, gg_xyz, gg_rr, gg_params, workspace, workspace_bytes, stream);
}

}  // extern "C"
