// A plain BF16 x BF16 -> FP32 GEMM on the tcgen05 tensor cores:
// D[M,N] = A[M,K] . B[K,N] with A row-major and B given transposed (Bt [N,K]
// row-major, i.e. K-major).  One CTA per 128-row tile; K is staged through
// shared memory in chunks of 64 in the core-matrix layout; the accumulator
// lives in TMEM and is read back with tcgen05.ld.  It checks the descriptor
// conventions the fused kernels rely on and serves plain library GEMMs.
#include "common.cuh"
#include "tc.cuh"

namespace dpgb {
namespace {

constexpr int kKC = 64;  // K chunk staged per MMA batch

__global__ void __launch_bounds__(128)
tc_gemm_kernel(float* __restrict__ D, const __nv_bfloat16* __restrict__ A, const __nv_bfloat16* __restrict__ Bt,
               int M, int N, int K, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  unsigned char* sA = smem;                       // 128 x kKC bf16 = 16 KB
  unsigned char* sB = smem + 128 * kKC * 2;       // N x kKC bf16
  const int m0 = blockIdx.x * 128;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t ncols = 32;
  while ((int)ncols < N) ncols <<= 1;
  if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
  if (threadIdx.x == 0) tc::mbar_init(&bar, 1);
  __syncthreads();
  tc::fence_after();
  const uint32_t tbase = tmem_base;
  const uint32_t idesc = tc::idesc_bf16_f32(128, N);
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = 0; k0 < K && ok; k0 += kKC) {
    const int kc = min(kKC, K - k0);  // multiple of 16
    // stage A rows [m0, m0+128) and Bt rows [0, N) of this K chunk; 16-byte chunks
    const int achunks = 128 * (kc / 8);
    for (int q = threadIdx.x; q < achunks; q += blockDim.x) {
      const int r = q / (kc / 8), c8 = q % (kc / 8);
      uint4 v = make_uint4(0, 0, 0, 0);
      if (m0 + r < M) v = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * K + k0 + c8 * 8);
      *reinterpret_cast<uint4*>(sA + tc::cm_offset(r, c8 * 8, kc)) = v;
    }
    const int bchunks = N * (kc / 8);
    for (int q = threadIdx.x; q < bchunks; q += blockDim.x) {
      const int r = q / (kc / 8), c8 = q % (kc / 8);
      const uint4 v = *reinterpret_cast<const uint4*>(Bt + (size_t)r * K + k0 + c8 * 8);
      *reinterpret_cast<uint4*>(sB + tc::cm_offset(r, c8 * 8, kc)) = v;
    }
    tc::fence_async_smem();
    __syncthreads();
    tc::fence_after();
    if (threadIdx.x == 0) {
      const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
      for (int ks = 0; ks < kc / 16; ++ks) {
        const uint64_t ad = tc::smem_desc(a0 + ks * 256, 128, (kc / 8) * 128);
        const uint64_t bd = tc::smem_desc(b0 + ks * 256, 128, (kc / 8) * 128);
        tc::mma_bf16(tbase, ad, bd, idesc, (k0 > 0 || ks > 0) ? 1u : 0u);
      }
      tc::mma_commit(&bar);
    }
    ok = tc::mbar_wait(&bar, phase, err);
    phase ^= 1;
    tc::fence_after();
    ok = __syncthreads_and(ok) != 0;  // uniform across the CTA
  }
  if (ok) {
    // warp w reads TMEM lanes 32w..32w+31 = tile rows
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(tc::taddr(tbase, warp * 32, c0), v);
      tc::tmem_ld_wait();
      if (row < M)
#pragma unroll
        for (int i = 0; i < 16; ++i) D[(size_t)row * N + c0 + i] = v[i];
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, ncols);
}

}  // namespace
}  // namespace dpgb

using namespace dpgb;

extern "C" int dpgb_tc_gemm_bf16(float* D, const void* A, const void* Bt, int M, int N, int K, void* stream) {
  clear_error();
  if (M <= 0 || N < 16 || N > 256 || N % 16 || K <= 0 || K % 16 || !D || !A || !Bt)
    return fail(DPGB_EINVAL, "tc_gemm_bf16: M > 0, N in 16..256 (multiple of 16), K multiple of 16");
  cudaStream_t st = as_stream(stream);
  DeviceBuffer ws;
  DPGB_TRY(ws.alloc(sizeof(int) * 4));
  DPGB_CUDA(cudaMemsetAsync(ws.ptr, 0, sizeof(int) * 4, st));
  const size_t smem = (size_t)(128 + N) * kKC * 2;
  DPGB_CUDA(cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  tc_gemm_kernel<<<ceil_div(M, 128), 128, smem, st>>>(D, reinterpret_cast<const __nv_bfloat16*>(A),
                                                       reinterpret_cast<const __nv_bfloat16*>(Bt), M, N, K,
                                                       ws.as<int>());
  DPGB_TRY(check_launch("tc_gemm_bf16"));
  int h = 0;
  DPGB_CUDA(cudaMemcpyAsync(&h, ws.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  DPGB_CUDA(cudaStreamSynchronize(st));
  if (h) return fail(DPGB_ETIMEOUT, "tc_gemm_bf16: the MMA completion wait timed out");
  return DPGB_OK;
}
