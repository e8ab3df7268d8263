// tabulate_fusion_se_a: the compressed se_e2_a embedding (a fifth-order
// polynomial per neuron per table interval) fused with the G^T R~ contraction,
// plus its first and second derivatives.
//
// Semantics follow source/lib/src/tabulate.cc:45-449 (locate_xx, polynomial5,
// the sorted-padding fold at the first trailing padding slot) for NDESCRPT=4.
// GPU layout: one CTA per (atom, 128-neuron chunk); the CTA's four warps split
// the neighbours round-robin, each lane owns up to four neurons, so the table
// row of one interval is read as contiguous 6-coefficient groups; partial
// sums are reduced across warps in shared memory (no atomics, deterministic).
#include "common.cuh"

namespace dpgb {
namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kNeuronChunk = 128;  // neurons per CTA (4 per lane)

template <typename T>
struct TabInfo {
  T lower, upper, mx, s0, s1;
  int first;   // int((upper - lower) / stride0)
  int hi_idx;  // table index used beyond max
  T hi_xx;     // local coordinate used beyond max
};

template <typename T>
__device__ __forceinline__ void locate(const TabInfo<T>& ti, T& xx, int& idx, T& delta) {
  const T orig = xx;
  delta = (T)0;
  if (xx < ti.lower) {
    idx = 0;
    xx = (T)0;
    delta = orig - ti.lower;
  } else if (xx < ti.upper) {
    idx = (int)((xx - ti.lower) / ti.s0);
    xx -= (idx * ti.s0 + ti.lower);
  } else if (xx < ti.mx) {
    idx = ti.first + (int)((xx - ti.upper) / ti.s1);
    xx -= ((idx - ti.first) * ti.s1 + ti.upper);
  } else {
    idx = ti.hi_idx;
    xx = ti.hi_xx;
    delta = orig - ti.mx;
  }
}

template <typename T>
struct Coef {
  T a0, a1, a2, a3, a4, a5;
};

__device__ __forceinline__ Coef<double> load_coef(const double* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  double2 x = __ldg(q), y = __ldg(q + 1), z = __ldg(q + 2);
  return {x.x, x.y, y.x, y.y, z.x, z.y};
}
__device__ __forceinline__ Coef<float> load_coef(const float* p) {
  const float2* q = reinterpret_cast<const float2*>(p);
  float2 x = __ldg(q), y = __ldg(q + 1), z = __ldg(q + 2);
  return {x.x, x.y, y.x, y.y, z.x, z.y};
}

template <typename T>
__device__ __forceinline__ T poly5(const Coef<T>& c, T x) {
  return c.a0 + (c.a1 + (c.a2 + (c.a3 + (c.a4 + c.a5 * x) * x) * x) * x) * x;
}
template <typename T>
__device__ __forceinline__ T poly5_grad(const Coef<T>& c, T x) {
  return c.a1 + ((T)2 * c.a2 + ((T)3 * c.a3 + ((T)4 * c.a4 + (T)5 * c.a5 * x) * x) * x) * x;
}

// First slot of the row that triggers the sorted-padding fold, or nnei.
template <typename T>
__device__ int fold_slot(const T* em_x_row, const T* em_row, int nnei, int is_sorted, int* s_red) {
  int best = nnei;
  if (is_sorted) {
    const T ago = em_x_row[nnei - 1];
    for (int jj = threadIdx.x; jj < nnei; jj += blockDim.x) {
      const T* ll = em_row + (size_t)jj * 4;
      if (em_x_row[jj] == ago && ll[1] == (T)0 && ll[2] == (T)0 && ll[3] == (T)0) {
        best = min(best, jj);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = best;
  __syncthreads();
  int r = s_red[0];
  for (int w = 1; w < kWarps; ++w) r = min(r, s_red[w]);
  __syncthreads();
  return r;
}

// out[i, m, n] = sum_j scale_j * poly(x_j)[n] * em[i, j, m]   (forward), or
// dz_dy[i, m, n] = sum_j scale_j * (var * hh[m] + dz_xx * var' * em[m])
// (second derivative), selected by GRADGRAD.
template <typename T, bool GRADGRAD>
__global__ void __launch_bounds__(kThreads)
tab_accumulate_kernel(T* __restrict__ out, const T* __restrict__ table, TabInfo<T> ti,
                      const T* __restrict__ em_x, const T* __restrict__ em,
                      const T* __restrict__ dz_x, const T* __restrict__ dz_em, int nnei,
                      int nl, int is_sorted) {
  __shared__ int s_red[kWarps];
  __shared__ T s_acc[kWarps][4][kNeuronChunk];
  const int ii = blockIdx.x;
  const int n0 = blockIdx.y * kNeuronChunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const T* ex = em_x + (size_t)ii * nnei;
  const T* erow = em + (size_t)ii * nnei * 4;
  const int jb = fold_slot(ex, erow, nnei, is_sorted, s_red);
  T acc[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int m = 0; m < 4; ++m) acc[k][m] = (T)0;
  const int jend = min(jb + 1, nnei);
  for (int jj = warp; jj < jend; jj += kWarps) {
    T xx = ex[jj];
    int idx;
    T delta;
    locate(ti, xx, idx, delta);
    const T scale = (jj == jb) ? (T)(nnei - jj) : (T)1;
    T ll[4], hh[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) ll[m] = erow[(size_t)jj * 4 + m];
    T dzx = (T)0;
    if (GRADGRAD) {
#pragma unroll
      for (int m = 0; m < 4; ++m) hh[m] = dz_em[((size_t)ii * nnei + jj) * 4 + m];
      dzx = dz_x[(size_t)ii * nnei + jj];
    }
    const T* trow = table + (size_t)idx * nl * 6;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int n = n0 + lane + 32 * k;
      if (n < nl && n < n0 + kNeuronChunk) {
        const Coef<T> c = load_coef(trow + 6 * (size_t)n);
        const T g = poly5_grad(c, xx);
        const T var = poly5(c, xx) + g * delta;
        if (GRADGRAD) {
#pragma unroll
          for (int m = 0; m < 4; ++m) acc[k][m] += scale * (var * hh[m] + dzx * g * ll[m]);
        } else {
          const T sv = scale * var;
#pragma unroll
          for (int m = 0; m < 4; ++m) acc[k][m] += sv * ll[m];
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int m = 0; m < 4; ++m) s_acc[warp][m][lane + 32 * k] = acc[k][m];
  __syncthreads();
  for (int q = threadIdx.x; q < 4 * kNeuronChunk; q += kThreads) {
    const int m = q / kNeuronChunk, nn = q % kNeuronChunk;
    const int n = n0 + nn;
    if (n < nl) {
      T s = s_acc[0][m][nn];
#pragma unroll
      for (int w = 1; w < kWarps; ++w) s += s_acc[w][m][nn];
      out[((size_t)ii * 4 + m) * nl + n] = s;
    }
  }
}

// dy_dem_x[i, j] = sum_n var'_n(x_j) (em_j . dy[:, n]) * scale,
// dy_dem[i, j, m] = sum_n var_n(x_j) dy[m, n] * scale; zero past the fold.
template <typename T>
__global__ void __launch_bounds__(kThreads)
tab_grad_kernel(T* __restrict__ dy_dem_x, T* __restrict__ dy_dem, const T* __restrict__ table,
                TabInfo<T> ti, const T* __restrict__ em_x, const T* __restrict__ em,
                const T* __restrict__ dy, int nnei, int nl, int is_sorted) {
  extern __shared__ unsigned char s_raw[];
  T* s_dy = reinterpret_cast<T*>(s_raw);  // [4][nl]
  __shared__ int s_red[kWarps];
  const int ii = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = threadIdx.x; q < 4 * nl; q += kThreads) s_dy[q] = dy[(size_t)ii * 4 * nl + q];
  const T* ex = em_x + (size_t)ii * nnei;
  const T* erow = em + (size_t)ii * nnei * 4;
  const int jb = fold_slot(ex, erow, nnei, is_sorted, s_red);  // also syncs s_dy
  for (int jj = warp; jj < nnei; jj += kWarps) {
    T g_sum = (T)0, d_sum[4] = {(T)0, (T)0, (T)0, (T)0};
    if (jj <= jb) {
      T xx = ex[jj];
      int idx;
      T delta;
      locate(ti, xx, idx, delta);
      T ll[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) ll[m] = erow[(size_t)jj * 4 + m];
      const T* trow = table + (size_t)idx * nl * 6;
      for (int n = lane; n < nl; n += 32) {
        const Coef<T> c = load_coef(trow + 6 * (size_t)n);
        const T g = poly5_grad(c, xx);
        const T res = poly5(c, xx) + g * delta;
        T rr[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) rr[m] = s_dy[m * nl + n];
        const T dot = ll[0] * rr[0] + ll[1] * rr[1] + ll[2] * rr[2] + ll[3] * rr[3];
        g_sum += g * dot;
#pragma unroll
        for (int m = 0; m < 4; ++m) d_sum[m] += res * rr[m];
      }
      g_sum = warp_sum(g_sum);
#pragma unroll
      for (int m = 0; m < 4; ++m) d_sum[m] = warp_sum(d_sum[m]);
      if (jj == jb) {
        const T sc = (T)(nnei - jj);
        g_sum *= sc;
#pragma unroll
        for (int m = 0; m < 4; ++m) d_sum[m] *= sc;
      }
    }
    if (lane == 0) {
      dy_dem_x[(size_t)ii * nnei + jj] = g_sum;
#pragma unroll
      for (int m = 0; m < 4; ++m) dy_dem[((size_t)ii * nnei + jj) * 4 + m] = d_sum[m];
    }
  }
}

template <typename T>
int make_info(const T* h, TabInfo<T>& ti) {
  if (h == nullptr) return fail(DPGB_EINVAL, "table_info must be a host array of 6");
  ti.lower = h[0];
  ti.upper = h[1];
  ti.mx = h[2];
  ti.s0 = h[3];
  ti.s1 = h[4];
  if (!(ti.s0 > (T)0) || !(ti.s1 > (T)0)) return fail(DPGB_EINVAL, "table strides must be positive");
  // locate_high_tail_xx (tabulate.cc:21-30), evaluated once on the host
  ti.first = (int)((ti.upper - ti.lower) / ti.s0);
  const T bxx = std::nextafter(ti.mx, ti.lower);
  ti.hi_idx = ti.first + (int)((bxx - ti.upper) / ti.s1);
  ti.hi_xx = ti.mx - ((ti.hi_idx - ti.first) * ti.s1 + ti.upper);
  return DPGB_OK;
}

template <typename T>
int check_common(const T* table, const T* em_x, const T* em, int nloc, int nnei, int nl) {
  if (nloc < 0 || nnei < 0 || nl <= 0) return fail(DPGB_EINVAL, "tabulate_fusion_se_a: bad sizes");
  if (nl > 1024)
    return fail(DPGB_EINVAL, "tabulate_fusion_se_a: last_layer_size must not exceed 1024");
  if (nloc > 0 && nnei > 0 && (!table || !em_x || !em))
    return fail(DPGB_EINVAL, "tabulate_fusion_se_a: NULL device pointer");
  if ((reinterpret_cast<uintptr_t>(table) & 15) != 0)
    return fail(DPGB_EINVAL, "tabulate_fusion_se_a: table must be 16-byte aligned");
  return DPGB_OK;
}

template <typename T>
int tab_forward(T* out, const T* table, const T* info, const T* em_x, const T* em, int nloc,
                int nnei, int nl, int is_sorted, void* stream, const T* dz_x, const T* dz_em) {
  DPGB_TRY(check_common(table, em_x, em, nloc, nnei, nl));
  if (nloc == 0) return DPGB_OK;
  cudaStream_t st = as_stream(stream);
  if (nnei == 0) {
    DPGB_CUDA(cudaMemsetAsync(out, 0, sizeof(T) * (size_t)nloc * 4 * nl, st));
    return DPGB_OK;
  }
  TabInfo<T> ti;
  DPGB_TRY(make_info(info, ti));
  dim3 grid(nloc, ceil_div(nl, kNeuronChunk));
  if (dz_x)
    tab_accumulate_kernel<T, true><<<grid, kThreads, 0, st>>>(out, table, ti, em_x, em, dz_x, dz_em,
                                                              nnei, nl, is_sorted);
  else
    tab_accumulate_kernel<T, false><<<grid, kThreads, 0, st>>>(out, table, ti, em_x, em, nullptr,
                                                               nullptr, nnei, nl, is_sorted);
  return check_launch("tabulate_fusion_se_a");
}

template <typename T>
int tab_grad(T* dx, T* dem, const T* table, const T* info, const T* em_x, const T* em, const T* dy,
             int nloc, int nnei, int nl, int is_sorted, void* stream) {
  DPGB_TRY(check_common(table, em_x, em, nloc, nnei, nl));
  if (nloc == 0 || nnei == 0) return DPGB_OK;
  TabInfo<T> ti;
  DPGB_TRY(make_info(info, ti));
  const size_t smem = sizeof(T) * 4 * nl;
  tab_grad_kernel<T><<<nloc, kThreads, smem, as_stream(stream)>>>(dx, dem, table, ti, em_x, em, dy,
                                                                  nnei, nl, is_sorted);
  return check_launch("tabulate_fusion_se_a_grad");
}

}  // namespace
}  // namespace dpgb

using namespace dpgb;

extern "C" {

int dpgb_tabulate_fusion_se_a_f64(double* out, const double* table, const double* info,
                                  const double* em_x, const double* em, int nloc, int nnei,
                                  int nl, int is_sorted, void* stream) {
  clear_error();
  return tab_forward<double>(out, table, info, em_x, em, nloc, nnei, nl, is_sorted, stream,
                             nullptr, nullptr);
}
int dpgb_tabulate_fusion_se_a_f32(float* out, const float* table, const float* info,
                                  const float* em_x, const float* em, int nloc, int nnei, int nl,
                                  int is_sorted, void* stream) {
  clear_error();
  return tab_forward<float>(out, table, info, em_x, em, nloc, nnei, nl, is_sorted, stream,
                            nullptr, nullptr);
}
int dpgb_tabulate_fusion_se_a_grad_f64(double* dx, double* dem, const double* table,
                                       const double* info, const double* em_x, const double* em,
                                       const double* dy, int nloc, int nnei, int nl,
                                       int is_sorted, void* stream) {
  clear_error();
  return tab_grad<double>(dx, dem, table, info, em_x, em, dy, nloc, nnei, nl, is_sorted, stream);
}
int dpgb_tabulate_fusion_se_a_grad_f32(float* dx, float* dem, const float* table,
                                       const float* info, const float* em_x, const float* em,
                                       const float* dy, int nloc, int nnei, int nl, int is_sorted,
                                       void* stream) {
  clear_error();
  return tab_grad<float>(dx, dem, table, info, em_x, em, dy, nloc, nnei, nl, is_sorted, stream);
}
int dpgb_tabulate_fusion_se_a_grad_grad_f64(double* dz_dy, const double* table,
                                            const double* info, const double* em_x,
                                            const double* em, const double* dz_x,
                                            const double* dz_em, int nloc, int nnei, int nl,
                                            int is_sorted, void* stream) {
  clear_error();
  if (nloc > 0 && nnei > 0 && (!dz_x || !dz_em))
    return fail(DPGB_EINVAL, "tabulate_fusion_se_a_grad_grad: NULL cotangent");
  return tab_forward<double>(dz_dy, table, info, em_x, em, nloc, nnei, nl, is_sorted, stream,
                             dz_x, dz_em);
}
int dpgb_tabulate_fusion_se_a_grad_grad_f32(float* dz_dy, const float* table, const float* info,
                                            const float* em_x, const float* em, const float* dz_x,
                                            const float* dz_em, int nloc, int nnei, int nl,
                                            int is_sorted, void* stream) {
  clear_error();
  if (nloc > 0 && nnei > 0 && (!dz_x || !dz_em))
    return fail(DPGB_EINVAL, "tabulate_fusion_se_a_grad_grad: NULL cotangent");
  return tab_forward<float>(dz_dy, table, info, em_x, em, nloc, nnei, nl, is_sorted, stream, dz_x,
                            dz_em);
}

}  // extern "C"
