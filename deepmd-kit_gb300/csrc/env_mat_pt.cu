// prod_env_mat in the PyTorch semantics (deepmd/pt/model/descriptor/env_mat.py:18-119)
// in FP64 or FP32, with its first and second derivatives with respect to the
// extended coordinates, written out by hand.
//
// Per kept pair, d = r_j - r_i, L = |d| (the reference's torch.linalg.norm,
// sqrt(fma(z,z,fma(y,y,x*x))) on the host), Lp = L + protection:
//   e0 = 1/Lp, e_{1..3} = d / Lp^2, w = s(clamp(L, rs, rc)), em = e * w,
//   out = (em - avg) / std; diff = d; sw = w.  Padding (j < 0 or j >= nall):
//   em = 0, diff = 0, sw = 0, out = -avg / std, no gradient.
// With ge = g_out / std, S = ge[1..3].d, B(L) = ge0 (e0' w + e0 w') + g_sw w',
// K(L) = h' w + h w' (h = Lp^-2), the pair gradient is
//   dL/dd = g_diff + (B + S K) d / L + w h ge[1..3],
// and along a direction delta = u_j - u_i the double backward needs
//   JVP:  d(em)(delta) = e_dot w + e w_dot, with L_dot = d.delta / L;
//   HVP:  grad_d <dL/dd, delta> = (delta/L - (d.delta) d / L^3)(B + S K)
//         + L_dot ((B' + S K') d/L + K ge[1..3]) + (ge[1..3].delta)(w h)' d/L.
// Pair terms reach atoms through the sorted transpose of the list (centre
// gets minus the sum of its row, neighbour plus the sum of its column):
// no atomics, reproducible run to run.
#include <vector>

#include "nlist.cuh"

namespace dpgb {
namespace {

template <typename T>
__device__ __forceinline__ T norm3(const T d[3]);
template <>
__device__ __forceinline__ double norm3<double>(const double d[3]) {
  return sqrt(fma(d[2], d[2], fma(d[1], d[1], d[0] * d[0])));
}
template <>
__device__ __forceinline__ float norm3<float>(const float d[3]) {
  return sqrtf(fmaf(d[2], d[2], fmaf(d[1], d[1], d[0] * d[0])));
}

// switch s(L) and its first two derivatives in L (clamped outside [rmin, rmax])
template <typename T>
__device__ __forceinline__ void switch_d2(T L, T rmin, T rmax, T& w, T& w1, T& w2) {
  const T xx = L < rmin ? rmin : (L > rmax ? rmax : L);
  const T width = rmax - rmin;
  const T uu = (xx - rmin) / width;
  const T uu2 = uu * uu;
  w = uu2 * uu * (T(-6) * uu2 + T(15) * uu - T(10)) + T(1);
  if (L >= rmin && L <= rmax) {
    const T um = uu - T(1);
    w1 = T(-30) * uu2 * um * um / width;
    w2 = T(-60) * uu * (T(2) * uu - T(1)) * um / (width * width);
  } else {
    w1 = T(0);
    w2 = T(0);
  }
}

struct PairRef {
  int valid;
  int jj;  // slot
  int ti;
};

template <typename T>
__device__ __forceinline__ PairRef pair_of(long long q, const T* __restrict__ coord, const int* __restrict__ atype,
                                           const int* __restrict__ nlist, int nloc, int nall, int nnei, T d[3]) {
  PairRef r;
  const long long row = q / nnei;
  r.jj = (int)(q - row * nnei);
  const int f = (int)(row / nloc), i = (int)(row - (long long)f * nloc);
  const T* cf = coord + (size_t)f * nall * 3;
  r.ti = atype[(size_t)f * nloc + i];  // local types [nf, nloc]
  if (r.ti < 0) r.ti = 0;
  int j = nlist[q];
  r.valid = j >= 0 && j < nall;
  d[0] = d[1] = d[2] = T(0);
  if (r.valid)
#pragma unroll
    for (int k = 0; k < 3; ++k) d[k] = cf[3 * j + k] - cf[3 * i + k];
  return r;
}

template <typename T>
__global__ void env_fwd_kernel(T* __restrict__ em, T* __restrict__ diff, T* __restrict__ swo,
                               const int* __restrict__ nlist, const T* __restrict__ coord,
                               const int* __restrict__ atype, const T* __restrict__ avg, const T* __restrict__ std,
                               int nf, int nloc, int nall, int nnei, T rmin, T rmax, T prot) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nf * nloc * nnei) return;
  T d[3];
  const PairRef pr = pair_of(q, coord, atype, nlist, nloc, nall, nnei, d);
  T e4[4] = {T(0), T(0), T(0), T(0)}, w = T(0);
  if (pr.valid) {
    const T L = norm3(d);
    const T Lp = L + prot;
    T w1, w2;
    switch_d2(L, rmin, rmax, w, w1, w2);
    const T l2 = Lp * Lp;
    e4[0] = T(1) / Lp * w;
#pragma unroll
    for (int k = 0; k < 3; ++k) e4[1 + k] = d[k] / l2 * w;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) diff[3 * q + k] = d[k];
  swo[q] = w;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const size_t a = ((size_t)pr.ti * nnei + pr.jj) * 4 + c;
    em[4 * q + c] = (e4[c] - avg[a]) / std[a];
  }
}

// per-pair scalars shared by the backward and the double backward
template <typename T>
struct PairDer {
  T L, Lp, w, w1, w2, ge[4], S, B, K, Bp, Kp, wh, whp;
};

template <typename T>
__device__ __forceinline__ void pair_der(const T d[3], const T* go, const T* gsw, long long q, const T* __restrict__ std,
                                         const PairRef& pr, int nnei, T rmin, T rmax, T prot, PairDer<T>& P) {
  P.L = norm3(d);
  P.Lp = P.L + prot;
  switch_d2(P.L, rmin, rmax, P.w, P.w1, P.w2);
  const T iL = T(1) / P.Lp;
  const T f0 = iL, f0p = -iL * iL, f0pp = T(2) * iL * iL * iL;
  const T h = iL * iL, hp = T(-2) * iL * iL * iL, hpp = T(6) * iL * iL * iL * iL;
#pragma unroll
  for (int c = 0; c < 4; ++c) P.ge[c] = go ? go[4 * q + c] / std[((size_t)pr.ti * nnei + pr.jj) * 4 + c] : T(0);
  const T gs = gsw ? gsw[q] : T(0);
  P.S = P.ge[1] * d[0] + P.ge[2] * d[1] + P.ge[3] * d[2];
  P.B = P.ge[0] * (f0p * P.w + f0 * P.w1) + gs * P.w1;
  P.K = hp * P.w + h * P.w1;
  P.Bp = P.ge[0] * (f0pp * P.w + T(2) * f0p * P.w1 + f0 * P.w2) + gs * P.w2;
  P.Kp = hpp * P.w + T(2) * hp * P.w1 + h * P.w2;
  P.wh = P.w * h;
  P.whp = P.w1 * h + P.w * hp;
}

template <typename T>
__global__ void env_bwd_pair_kernel(T* __restrict__ pg, const T* __restrict__ go, const T* __restrict__ gdiff,
                                    const T* __restrict__ gsw, const int* __restrict__ nlist,
                                    const T* __restrict__ coord, const int* __restrict__ atype,
                                    const T* __restrict__ std, int nf, int nloc, int nall, int nnei, T rmin, T rmax,
                                    T prot) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nf * nloc * nnei) return;
  T d[3];
  const PairRef pr = pair_of(q, coord, atype, nlist, nloc, nall, nnei, d);
  T g[3] = {T(0), T(0), T(0)};
  if (pr.valid) {
    PairDer<T> P;
    pair_der(d, go, gsw, q, std, pr, nnei, rmin, rmax, prot, P);
    const T coef = (P.B + P.S * P.K) / P.L;
#pragma unroll
    for (int k = 0; k < 3; ++k) g[k] = (gdiff ? gdiff[3 * q + k] : T(0)) + coef * d[k] + P.wh * P.ge[1 + k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) pg[3 * q + k] = g[k];
}

template <typename T>
__global__ void env_bwd_bwd_pair_kernel(T* __restrict__ gg_em, T* __restrict__ gg_diff, T* __restrict__ gg_sw,
                                        T* __restrict__ pg, const T* __restrict__ u, const T* __restrict__ go,
                                        const T* __restrict__ gsw, const int* __restrict__ nlist,
                                        const T* __restrict__ coord, const int* __restrict__ atype,
                                        const T* __restrict__ std, int nf, int nloc, int nall, int nnei, T rmin,
                                        T rmax, T prot) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nf * nloc * nnei) return;
  T d[3];
  const PairRef pr = pair_of(q, coord, atype, nlist, nloc, nall, nnei, d);
  T jem[4] = {T(0), T(0), T(0), T(0)}, jd[3] = {T(0), T(0), T(0)}, jsw = T(0), hv[3] = {T(0), T(0), T(0)};
  if (pr.valid) {
    const long long row = q / nnei;
    const int f = (int)(row / nloc), i = (int)(row - (long long)f * nloc);
    const int j = nlist[q];
    const T* uf = u + (size_t)f * nall * 3;
    T dl[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dl[k] = uf[3 * j + k] - uf[3 * i + k];
    PairDer<T> P;
    pair_der(d, go, gsw, q, std, pr, nnei, rmin, rmax, prot, P);
    const T m = d[0] * dl[0] + d[1] * dl[1] + d[2] * dl[2];
    const T Ld = m / P.L;
    const T iL = T(1) / P.Lp;
    const T h = iL * iL, hp = T(-2) * iL * iL * iL;
    const T wd = P.w1 * Ld;
    // JVP of em, diff, sw
    const T e0 = iL, e0d = -iL * iL * Ld;
    const size_t a0 = ((size_t)pr.ti * nnei + pr.jj) * 4;
    jem[0] = (e0d * P.w + e0 * wd) / std[a0];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const T ek = d[k] * h, ekd = dl[k] * h + d[k] * hp * Ld;
      jem[1 + k] = (ekd * P.w + ek * wd) / std[a0 + 1 + k];
      jd[k] = dl[k];
    }
    jsw = wd;
    // HVP of the pair gradient along delta
    if (pg) {
      const T BSK = P.B + P.S * P.K;
      const T c2 = Ld * (P.Bp + P.S * P.Kp) / P.L;
      const T Pd = P.ge[1] * dl[0] + P.ge[2] * dl[1] + P.ge[3] * dl[2];
      const T c3 = Pd * P.whp / P.L;
      const T iL3 = T(1) / (P.L * P.L * P.L);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        hv[k] = (dl[k] / P.L - m * d[k] * iL3) * BSK + c2 * d[k] + Ld * P.K * P.ge[1 + k] + c3 * d[k];
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) gg_em[4 * q + c] = jem[c];
  if (gg_diff)
#pragma unroll
    for (int k = 0; k < 3; ++k) gg_diff[3 * q + k] = jd[k];
  if (gg_sw) gg_sw[q] = jsw;
  if (pg)
#pragma unroll
    for (int k = 0; k < 3; ++k) pg[3 * q + k] = hv[k];
}

__global__ void pair_keys_kernel(int* __restrict__ keys, const int* __restrict__ nlist, long long npair,
                                 long long per_frame, int nall) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int j = nlist[p];
  keys[p] = (j < 0 || j >= nall) ? -1 : (int)(j + (p / per_frame) * nall);
}

// out[f, j] = -sum over row (f, j)'s slots (j < nloc) + sum over pairs pointing at (f, j)
template <typename T>
__global__ void pair_gather_kernel(T* __restrict__ out, const T* __restrict__ pg, Transpose tr, int nloc, int nall,
                                   int nnei, int nf) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nf * nall) return;
  const int f = (int)(q / nall), j = (int)(q - (long long)f * nall);
  double acc[3] = {0.0, 0.0, 0.0};
  if (j < nloc) {
    const T* row = pg + ((size_t)f * nloc + j) * nnei * 3;
    for (int s = 0; s < nnei; ++s)
#pragma unroll
      for (int k = 0; k < 3; ++k) acc[k] -= (double)row[3 * s + k];
  }
  for (int t = tr.offsets[q]; t < tr.offsets[q + 1]; ++t) {
    const int p = tr.pairs[t];
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[k] += (double)pg[3 * (size_t)p + k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) out[3 * q + k] = (T)acc[k];
}

int check_sizes(int nf, int nloc, int nall, int nnei, double rcut, double rcut_smth, const char* who) {
  if (nf < 1 || nloc < 0 || nall < nloc || nnei < 1) return fail(DPGB_EINVAL, std::string(who) + ": bad sizes");
  if (!(rcut > rcut_smth)) return fail(DPGB_EINVAL, std::string(who) + ": rcut must exceed rcut_smth");
  if ((long long)nf * nall >= (1LL << 31) || (long long)nf * nloc * nnei >= (1LL << 31))
    return fail(DPGB_EINVAL, std::string(who) + ": too large");
  return DPGB_OK;
}

// gather pair vectors pg [npair, 3] (device) into out [nf, nall, 3]
template <typename T>
int gather_pairs(T* out, const T* pg, const int* nlist, int nf, int nloc, int nall, int nnei, cudaStream_t st,
                 const char* who) {
  const long long npair = (long long)nf * nloc * nnei;
  const long long nkeys = (long long)nf * nall;
  DeviceBuffer& ws = thread_scratch(0);  // done with before the status read below returns
  const size_t key_bytes = sizeof(int) * (size_t)npair;
  const size_t tr_bytes = transpose_workspace(npair, (int)nkeys);
  DPGB_TRY(ws.alloc(key_bytes + tr_bytes + sizeof(int) * kStatusSlots + 64));
  int* keys = ws.as<int>();
  int* status = keys + npair;
  void* trw = status + kStatusSlots;
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  if (npair > 0) {
    pair_keys_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(keys, nlist, npair, (long long)nloc * nnei, nall);
    DPGB_TRY(check_launch("pair_keys"));
  }
  Transpose tr;
  DPGB_TRY(launch_transpose(tr, keys, npair, (int)nkeys, 0, trw, status, st));
  pair_gather_kernel<T><<<ceil_div(nkeys, 256), 256, 0, st>>>(out, pg, tr, nloc, nall, nnei, nf);
  DPGB_TRY(check_launch("pair_gather"));
  int h[kStatusSlots];
  DPGB_TRY(read_status(status, st, h));  // keeps the workspace alive until the gather is done
  if (h[kStatusOverflow] > 0) return fail(DPGB_EOVERFLOW, std::string(who) + ": an atom appears in more than 2048 rows");
  return DPGB_OK;
}

template <typename T>
int env_fwd(T* em, T* diff, T* sw, const T* coord, const int* atype, const int* nlist, const T* avg, const T* std,
            int nf, int nloc, int nall, int nnei, double rcut, double rcut_smth, double prot, void* stream) {
  clear_error();
  DPGB_TRY(check_sizes(nf, nloc, nall, nnei, rcut, rcut_smth, "env_mat_pt"));
  if (!em || !diff || !sw || !coord || !atype || !nlist || !avg || !std) return fail(DPGB_EINVAL, "env_mat_pt: NULL pointer");
  const long long n = (long long)nf * nloc * nnei;
  if (n == 0) return DPGB_OK;
  env_fwd_kernel<T><<<ceil_div(n, 256), 256, 0, as_stream(stream)>>>(em, diff, sw, nlist, coord, atype, avg, std, nf,
                                                                       nloc, nall, nnei, (T)rcut_smth, (T)rcut, (T)prot);
  return check_launch("env_mat_pt");
}

template <typename T>
int env_bwd(T* g_coord, const T* g_em, const T* g_diff, const T* g_sw, const T* coord, const int* atype,
            const int* nlist, const T* std, int nf, int nloc, int nall, int nnei, double rcut, double rcut_smth,
            double prot, void* stream) {
  clear_error();
  DPGB_TRY(check_sizes(nf, nloc, nall, nnei, rcut, rcut_smth, "env_mat_pt_bwd"));
  if (!g_coord || !coord || !atype || !nlist || !std) return fail(DPGB_EINVAL, "env_mat_pt_bwd: NULL pointer");
  cudaStream_t st = as_stream(stream);
  const long long n = (long long)nf * nloc * nnei;
  DeviceBuffer& pgb = thread_scratch(1);  // read by the gather, which synchronises
  DPGB_TRY(pgb.alloc(sizeof(T) * 3 * (size_t)std::max<long long>(n, 1)));
  if (n > 0) {
    env_bwd_pair_kernel<T><<<ceil_div(n, 256), 256, 0, st>>>(pgb.as<T>(), g_em, g_diff, g_sw, nlist, coord, atype, std,
                                                             nf, nloc, nall, nnei, (T)rcut_smth, (T)rcut, (T)prot);
    DPGB_TRY(check_launch("env_mat_pt_bwd"));
  }
  return gather_pairs<T>(g_coord, pgb.as<T>(), nlist, nf, nloc, nall, nnei, st, "env_mat_pt_bwd");
}

template <typename T>
int env_bwd_bwd(T* gg_em, T* gg_diff, T* gg_sw, T* gg_coord, const T* u, const T* g_em, const T* g_diff,
                const T* g_sw, const T* coord, const int* atype, const int* nlist, const T* std, int nf, int nloc,
                int nall, int nnei, double rcut, double rcut_smth, double prot, void* stream) {
  (void)g_diff;  // the pair gradient is linear in g_diff: no curvature term
  clear_error();
  DPGB_TRY(check_sizes(nf, nloc, nall, nnei, rcut, rcut_smth, "env_mat_pt_bwd_bwd"));
  if (!gg_em || !u || !coord || !atype || !nlist || !std) return fail(DPGB_EINVAL, "env_mat_pt_bwd_bwd: NULL pointer");
  cudaStream_t st = as_stream(stream);
  const long long n = (long long)nf * nloc * nnei;
  DeviceBuffer& pgb = thread_scratch(1);  // used only with gg_coord, whose gather synchronises
  if (gg_coord) DPGB_TRY(pgb.alloc(sizeof(T) * 3 * (size_t)std::max<long long>(n, 1)));
  if (n > 0) {
    env_bwd_bwd_pair_kernel<T><<<ceil_div(n, 256), 256, 0, st>>>(gg_em, gg_diff, gg_sw, gg_coord ? pgb.as<T>() : nullptr,
                                                                 u, g_em, g_sw, nlist, coord, atype, std, nf, nloc,
                                                                 nall, nnei, (T)rcut_smth, (T)rcut, (T)prot);
    DPGB_TRY(check_launch("env_mat_pt_bwd_bwd"));
  }
  if (!gg_coord) return DPGB_OK;
  return gather_pairs<T>(gg_coord, pgb.as<T>(), nlist, nf, nloc, nall, nnei, st, "env_mat_pt_bwd_bwd");
}

}  // namespace
}  // namespace dpgb

using namespace dpgb;

extern "C" {

int dpgb_env_mat_pt2_f64(double* em, double* diff, double* sw, const double* coord_ext, const int* atype_ext,
                         const int* nlist, const double* avg, const double* std, int nf, int nloc, int nall, int nnei,
                         double rcut, double rcut_smth, double protection, void* stream) {
  return env_fwd<double>(em, diff, sw, coord_ext, atype_ext, nlist, avg, std, nf, nloc, nall, nnei, rcut, rcut_smth,
                         protection, stream);
}
int dpgb_env_mat_pt2_f32(float* em, float* diff, float* sw, const float* coord_ext, const int* atype_ext,
                         const int* nlist, const float* avg, const float* std, int nf, int nloc, int nall, int nnei,
                         double rcut, double rcut_smth, double protection, void* stream) {
  return env_fwd<float>(em, diff, sw, coord_ext, atype_ext, nlist, avg, std, nf, nloc, nall, nnei, rcut, rcut_smth,
                        protection, stream);
}

int dpgb_env_mat_pt_bwd_f64(double* g_coord, const double* g_em, const double* g_diff, const double* g_sw,
                            const double* coord_ext, const int* atype_ext, const int* nlist, const double* std, int nf,
                            int nloc, int nall, int nnei, double rcut, double rcut_smth, double protection,
                            void* stream) {
  return env_bwd<double>(g_coord, g_em, g_diff, g_sw, coord_ext, atype_ext, nlist, std, nf, nloc, nall, nnei, rcut,
                         rcut_smth, protection, stream);
}
int dpgb_env_mat_pt_bwd_f32(float* g_coord, const float* g_em, const float* g_diff, const float* g_sw,
                            const float* coord_ext, const int* atype_ext, const int* nlist, const float* std, int nf,
                            int nloc, int nall, int nnei, double rcut, double rcut_smth, double protection,
                            void* stream) {
  return env_bwd<float>(g_coord, g_em, g_diff, g_sw, coord_ext, atype_ext, nlist, std, nf, nloc, nall, nnei, rcut,
                        rcut_smth, protection, stream);
}

int dpgb_env_mat_pt_bwd_bwd_f64(double* gg_em, double* gg_diff, double* gg_sw, double* gg_coord, const double* u,
                                const double* g_em, const double* g_diff, const double* g_sw, const double* coord_ext,
                                const int* atype_ext, const int* nlist, const double* std, int nf, int nloc, int nall,
                                int nnei, double rcut, double rcut_smth, double protection, void* stream) {
  return env_bwd_bwd<double>(gg_em, gg_diff, gg_sw, gg_coord, u, g_em, g_diff, g_sw, coord_ext, atype_ext, nlist, std,
                             nf, nloc, nall, nnei, rcut, rcut_smth, protection, stream);
}
int dpgb_env_mat_pt_bwd_bwd_f32(float* gg_em, float* gg_diff, float* gg_sw, float* gg_coord, const float* u,
                                const float* g_em, const float* g_diff, const float* g_sw, const float* coord_ext,
                                const int* atype_ext, const int* nlist, const float* std, int nf, int nloc, int nall,
                                int nnei, double rcut, double rcut_smth, double protection, void* stream) {
  return env_bwd_bwd<float>(gg_em, gg_diff, gg_sw, gg_coord, u, g_em, g_diff, g_sw, coord_ext, atype_ext, nlist, std,
                            nf, nloc, nall, nnei, rcut, rcut_smth, protection, stream);
}

}  // extern "C"
