// Energy fitting net (deepmd/pt/model/task/fitting.py:734-899,
// deepmd/dpmodel/utils/network.py:935-1000) forward and input-gradient
// backward over the rows of one atom type, SIMT form (FP64 or FP32).
//
// Hidden layer l: Y_l = tanh(X W_l + b_l) [* idt_l] (+ X when widths match,
// + [X, X] when the width doubles); output e = Y_L w + b.  The backward pass
// produces dE/dD row by row for the descriptor backward.
#include "se_a.cuh"

namespace dpgb {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, kGemmThreads = 256;

template <typename T>
__device__ __forceinline__ T tanh_f(T x);
template <>
__device__ __forceinline__ double tanh_f<double>(double x) { return tanh(x); }
template <>
__device__ __forceinline__ float tanh_f<float>(float x) { return tanhf(x); }

enum EpiMode { kEpiStore = 0, kEpiFwd = 1, kEpiBwd = 2 };

template <typename T>
struct Epi {
  int mode;
  // forward
  const T* bias;
  const T* idt;
  const T* X;     // layer input (skip source), ld = ldx
  int ldx, nin;   // input width for the skip rule
  T* Y;           // layer output
  T* Tt;          // tanh values
  int ldy;
  // backward
  const T* dY;    // gradient of the layer output (skip source), ld = ld_dy
  int ld_dy, nout;  // output width of the layer being back-propagated
  T* dX;          // gradient of the layer input
  int ld_dx;
  const T* idt_lo;  // lower layer's timestep (NULL = 1)
  const T* T_lo;    // lower layer's tanh values (NULL: no dP output)
  int ld_tlo;
  T* dP_lo;         // dX * idt_lo * (1 - T_lo^2)
};

// C[M,N] = A[M,K] . B  with B [K,N] (TRANSB = false) or B [N,K] (TRANSB = true)
template <typename T, bool TRANSB>
__global__ void __launch_bounds__(kGemmThreads)
gemm_kernel(int M, int N, int K, const T* __restrict__ A, int lda, const T* __restrict__ B, int ldb,
            Epi<T> ep) {
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = (T)0;
  for (int k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int idx = t + e * kGemmThreads;
      const int r = idx >> 4, k = idx & 15;
      const int gm = m0 + r, gk = k0 + k;
      As[k][r] = (gm < M && gk < K) ? A[(size_t)gm * lda + gk] : (T)0;
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int idx = t + e * kGemmThreads;
      if (!TRANSB) {
        const int k = idx >> 6, n = idx & 63;
        const int gk = k0 + k, gn = n0 + n;
        Bs[k][n] = (gk < K && gn < N) ? __ldg(B + (size_t)gk * ldb + gn) : (T)0;
      } else {
        const int n = idx >> 4, k = idx & 15;
        const int gk = k0 + k, gn = n0 + n;
        Bs[k][n] = (gk < K && gn < N) ? __ldg(B + (size_t)gn * ldb + gk) : (T)0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx + 16 * j;
      if (n >= N) continue;
      const T v = acc[i][j];
      if (ep.mode == kEpiFwd) {
        const T tv = tanh_f<T>(v + ep.bias[n]);
        T y = ep.idt ? tv * ep.idt[n] : tv;
        if (N == ep.nin)
          y += ep.X[(size_t)m * ep.ldx + n];
        else if (N == 2 * ep.nin)
          y += ep.X[(size_t)m * ep.ldx + (n < ep.nin ? n : n - ep.nin)];
        ep.Y[(size_t)m * ep.ldy + n] = y;
        ep.Tt[(size_t)m * ep.ldy + n] = tv;
      } else if (ep.mode == kEpiBwd) {
        T dx = v;
        if (ep.dY) {
          if (ep.nout == N)
            dx += ep.dY[(size_t)m * ep.ld_dy + n];
          else if (ep.nout == 2 * N)
            dx += ep.dY[(size_t)m * ep.ld_dy + n] + ep.dY[(size_t)m * ep.ld_dy + n + N];
        }
        ep.dX[(size_t)m * ep.ld_dx + n] = dx;
        if (ep.T_lo) {
          const T tl = ep.T_lo[(size_t)m * ep.ld_tlo + n];
          ep.dP_lo[(size_t)m * ep.ld_dx + n] = dx * (ep.idt_lo ? ep.idt_lo[n] : (T)1) * ((T)1 - tl * tl);
        }
      } else {
        ep.dX[(size_t)m * ep.ld_dx + n] = v;
      }
    }
  }
}

// e[m] = Y[m] . w + b (one warp per row)
template <typename T>
__global__ void out_layer_kernel(double* __restrict__ e, const T* __restrict__ Y, int ldy, int K,
                                 const T* __restrict__ w, const T* __restrict__ b, int M) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= M) return;
  T s = (T)0;
  for (int k = lane; k < K; k += 32) s += Y[(size_t)warp * ldy + k] * w[k];
  s = warp_sum(s);
  if (lane == 0) e[warp] = (double)(s + b[0]);
}

// dY_L = w (broadcast), dP_L = w * idt_L * (1 - T_L^2)
template <typename T>
__global__ void out_grad_kernel(T* __restrict__ dY, T* __restrict__ dP, const T* __restrict__ Tt,
                                int ld, int K, const T* __restrict__ w, const T* __restrict__ idt,
                                int M) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)M * K) return;
  const int m = (int)(q / K), k = (int)(q % K);
  const T tv = Tt[(size_t)m * ld + k];
  dY[(size_t)m * ld + k] = w[k];
  dP[(size_t)m * ld + k] = w[k] * (idt ? idt[k] : (T)1) * ((T)1 - tv * tv);
}

template <typename T, bool TRANSB>
int gemm(int M, int N, int K, const T* A, int lda, const T* B, int ldb, const Epi<T>& ep, cudaStream_t st) {
  if (M <= 0 || N <= 0) return DPGB_OK;
  dim3 grid(ceil_div(N, BN), ceil_div(M, BM));
  gemm_kernel<T, TRANSB><<<grid, kGemmThreads, 0, st>>>(M, N, K, A, lda, B, ldb, ep);
  return check_launch("fitting_gemm");
}

}  // namespace

template <typename T>
int launch_fitting(const FitParams<T>& f, int type, int row0, int nrow, int nrows_total, const T* D,
                   T* dD, T* act, T* gbuf, double* e_sorted, double ener_bias, cudaStream_t st) {
  (void)ener_bias;
  if (nrow <= 0) return DPGB_OK;
  const int L = f.n_hidden;
  int maxw = 0;
  for (int l = 1; l <= L; ++l) maxw = maxw > f.width[l] ? maxw : f.width[l];
  const size_t plane = (size_t)nrows_total * maxw;
  auto Ybuf = [&](int l) { return act + (2 * (size_t)l) * plane + (size_t)row0 * maxw; };
  auto Tbuf = [&](int l) { return act + (2 * (size_t)l + 1) * plane + (size_t)row0 * maxw; };
  auto G = [&](int k) { return gbuf + (size_t)k * plane + (size_t)row0 * maxw; };
  const int dim = f.width[0];
  const T* Drow = D + (size_t)row0 * dim;
  T* dDrow = dD + (size_t)row0 * dim;
  // forward
  const T* in = Drow;
  int ldin = dim;
  for (int l = 0; l < L; ++l) {
    const int nin = f.width[l], nout = f.width[l + 1];
    Epi<T> ep{};
    ep.mode = kEpiFwd;
    ep.bias = f.b[l] + (size_t)type * nout;
    ep.idt = f.idt[l] ? f.idt[l] + (size_t)type * nout : nullptr;
    ep.X = in;
    ep.ldx = ldin;
    ep.nin = nin;
    ep.Y = Ybuf(l);
    ep.Tt = Tbuf(l);
    ep.ldy = maxw;
    DPGB_TRY((gemm<T, false>(nrow, nout, nin, in, ldin, f.W[l] + (size_t)type * nin * nout, nout, ep, st)));
    in = Ybuf(l);
    ldin = maxw;
  }
  const int wl = f.width[L];
  out_layer_kernel<T><<<ceil_div((long long)nrow * 32, 256), 256, 0, st>>>(
      e_sorted + row0, in, ldin, wl, f.w_out + (size_t)type * wl, f.b_out + type, nrow);
  DPGB_TRY(check_launch("fitting_out"));
  if (L == 0) return fail(DPGB_EINVAL, "fitting nets without hidden layers are not supported");
  // backward: buffers 0/1 hold (dY, dP) of the current layer, 2/3 the next
  int cur = 0;
  {
    const T* idt = f.idt[L - 1] ? f.idt[L - 1] + (size_t)type * wl : nullptr;
    out_grad_kernel<T><<<ceil_div((long long)nrow * wl, 256), 256, 0, st>>>(
        G(0), G(1), Tbuf(L - 1), maxw, wl, f.w_out + (size_t)type * wl, idt, nrow);
    DPGB_TRY(check_launch("fitting_out_grad"));
  }
  for (int l = L - 1; l >= 0; --l) {
    const int nin = f.width[l], nout = f.width[l + 1];
    T* dY = G(cur);
    T* dP = G(cur + 1);
    Epi<T> ep{};
    ep.mode = kEpiBwd;
    ep.nout = nout;
    // the skip term exists only when the layer has one (widths equal / doubled)
    ep.dY = (nout == nin || nout == 2 * nin) ? dY : nullptr;
    ep.ld_dy = maxw;
    if (l > 0) {
      const int nxt = cur ^ 2;
      ep.dX = G(nxt);
      ep.ld_dx = maxw;
      ep.T_lo = Tbuf(l - 1);
      ep.ld_tlo = maxw;
      ep.idt_lo = f.idt[l - 1] ? f.idt[l - 1] + (size_t)type * nin : nullptr;
      ep.dP_lo = G(nxt + 1);
      DPGB_TRY((gemm<T, true>(nrow, nin, nout, dP, maxw, f.W[l] + (size_t)type * nin * nout, nout, ep, st)));
      cur = nxt;
    } else {
      ep.dX = dDrow;
      ep.ld_dx = dim;
      DPGB_TRY((gemm<T, true>(nrow, nin, nout, dP, maxw, f.W[l] + (size_t)type * nin * nout, nout, ep, st)));
    }
  }
  return DPGB_OK;
}

template int launch_fitting<double>(const FitParams<double>&, int, int, int, int, const double*, double*,
                                    double*, double*, double*, double, cudaStream_t);
template int launch_fitting<float>(const FitParams<float>&, int, int, int, int, const float*, float*, float*,
                                   float*, double*, double, cudaStream_t);

}  // namespace dpgb
