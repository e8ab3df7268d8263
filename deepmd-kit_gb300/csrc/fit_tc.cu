// Tensor-core (tcgen05) energy fitting net for the mixed-precision DeepPot:
// forward tanh layers, the output layer and the input-gradient backward
// (dE/dD) as BF16 GEMMs with FP32 TMEM accumulators and fused epilogues
// (deepmd/pt/model/task/fitting.py:734-899 semantics; hidden layer
// y = tanh(x W + b) * idt (+ x when the widths match)).
//
// One CTA computes a 128-row x (<= 256)-column tile; K is staged in chunks of
// 64 through two shared-memory buffers so that the loads of chunk k+1 overlap
// the MMAs of chunk k.
#include "fit_tc.cuh"
#include "tc.cuh"

namespace dpgb {
namespace {

constexpr int kKC = 64;
constexpr int kNT = 256;

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// stage rows [0, nrows) x K-chunk [k0, k0+kc) of a row-major bf16 matrix
__device__ __forceinline__ void stage(unsigned char* dst, const __nv_bfloat16* src, int ld, int nrows, int rows_valid,
                                      int k0, int kc) {
  const int per = kc / 8;
  for (int q = threadIdx.x; q < nrows * per; q += blockDim.x) {
    const int r = q / per, c8 = q - r * per;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (r < rows_valid) v = __ldg(reinterpret_cast<const uint4*>(src + (size_t)r * ld + k0 + c8 * 8));
    *reinterpret_cast<uint4*>(dst + tc::cm_offset(r, c8 * 8, kc)) = v;
  }
}

__global__ void __launch_bounds__(128)
fit_gemm_kernel(FitGemm g, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar[2];
  __shared__ uint32_t s_tmem;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * 128;
  const int n0 = blockIdx.y * kNT;
  const int nt = min(kNT, g.N - n0);  // multiple of 16
  const int rows_valid = min(128, g.M - m0);
  unsigned char* sA[2] = {smem, smem + 128 * kKC * 2};
  unsigned char* sB[2] = {smem + 2 * 128 * kKC * 2, smem + 2 * 128 * kKC * 2 + kNT * kKC * 2};
  if (warp == 0) tc::tmem_alloc(&s_tmem, 256);
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
  }
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = s_tmem;
  const uint32_t idesc = tc::idesc_bf16_f32(128, nt);
  const __nv_bfloat16* A = g.A + (size_t)m0 * g.lda;
  const __nv_bfloat16* B = g.B + (size_t)n0 * g.K;
  uint32_t phase[2] = {0, 0};
  bool ok = true;
  const int nchunk = (g.K + kKC - 1) / kKC;
  for (int i = 0; i < nchunk; ++i) {
    const int b = i & 1;
    const int k0 = i * kKC, kc = min(kKC, g.K - k0);
    if (i >= 2) {  // the MMAs of chunk i-2 read this buffer
      ok = tc::mbar_wait(&bar[b], phase[b], err) && ok;
      phase[b] ^= 1;
    }
    stage(sA[b], A, g.lda, 128, rows_valid, k0, kc);
    stage(sB[b], B, g.K, nt, nt, k0, kc);
    tc::fence_async_smem();
    __syncthreads();
    tc::fence_after();
    if (threadIdx.x == 0) {
      const uint32_t a0 = tc::smem_u32(sA[b]), b0 = tc::smem_u32(sB[b]);
      const uint32_t sbo = (uint32_t)(kc / 8) * 128;
      for (int ks = 0; ks < kc / 16; ++ks)
        tc::mma_bf16(tbase, tc::smem_desc(a0 + ks * 256, 128, sbo), tc::smem_desc(b0 + ks * 256, 128, sbo), idesc,
                     (i > 0 || ks > 0) ? 1u : 0u);
      tc::mma_commit(&bar[b]);
    }
  }
  // drain: the last commit covers every MMA
  {
    const int last = (nchunk - 1) & 1;
    if (nchunk >= 2) {
      ok = tc::mbar_wait(&bar[last ^ 1], phase[last ^ 1], err) && ok;
    }
    ok = tc::mbar_wait(&bar[last], phase[last], err) && ok;
  }
  tc::fence_after();
  ok = __syncthreads_and(ok) != 0;
  if (ok) {
    const int r = warp * 32 + lane;
    const int m = m0 + r;
    const bool valid = r < rows_valid;
    double e_acc = 0.0;
    for (int c0 = 0; c0 < nt; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tc::taddr(tbase, warp * 32, c0), v);
      tc::tmem_ld_wait();
      if (!valid) continue;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int n = n0 + c0 + i;
        const float acc = v[i];
        if (g.mode == kFitFwd || g.mode == kFitFwdLast) {
          const float tv = tanh_fast(acc + g.bias[n]);
          float y = g.idt ? tv * g.idt[n] : tv;
          if (g.skip) y += g.Xs[(size_t)m * g.ldxs + n];
          if (g.mode == kFitFwd) {
            g.Yf[(size_t)m * g.ldy + n] = y;
            g.Yb[(size_t)m * g.ldy + n] = __float2bfloat16_rn(y);
            g.Tt[(size_t)m * g.ldy + n] = tv;
          } else {
            e_acc += (double)y * (double)g.w_out[n];
            const float dp = g.w_out[n] * (g.idt ? g.idt[n] : 1.f) * (1.f - tv * tv);
            g.dPb[(size_t)m * g.ldy + n] = __float2bfloat16_rn(dp);
          }
        } else if (g.mode == kFitBwd) {
          float dx = acc;
          if (g.dYup) dx += g.dYup[(size_t)m * g.lddyup + n];
          if (g.dXf) g.dXf[(size_t)m * g.ldy + n] = dx;
          const float tl = g.T_lo[(size_t)m * g.ldy + n];
          const float dp = dx * (g.idt_lo ? g.idt_lo[n] : 1.f) * (1.f - tl * tl);
          g.dPb[(size_t)m * g.ldy + n] = __float2bfloat16_rn(dp);
        } else {
          g.out[(size_t)m * g.ldo + n] = acc;
        }
      }
    }
    if (g.mode == kFitFwdLast && valid) g.e_out[m] = e_acc + (double)g.b_out;
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

}  // namespace

int fit_tc_eligible(const dpgb_se_a_desc& d) {
  if (d.dim_descrpt % 16) return 0;
  int nin = d.dim_descrpt;
  for (int l = 0; l < d.n_fit; ++l) {
    const int w = d.fit_neuron[l];
    if (w % 16 || w > 256) return 0;
    if (w == 2 * nin) return 0;  // the doubling skip is not fused here
    nin = w;
  }
  return d.n_fit >= 1;
}

int launch_fit_gemm(const FitGemm& g, int* err, cudaStream_t st) {
  if (g.M <= 0) return DPGB_OK;
  const size_t smem = (size_t)2 * (128 + kNT) * kKC * 2;
  static bool attr = false;
  if (!attr) {
    DPGB_CUDA(cudaFuncSetAttribute(fit_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  dim3 grid(ceil_div(g.M, 128), ceil_div(g.N, kNT));
  fit_gemm_kernel<<<grid, 128, smem, st>>>(g, err);
  return check_launch("fit_gemm");
}

}  // namespace dpgb
