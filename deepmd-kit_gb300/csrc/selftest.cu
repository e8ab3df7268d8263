// Self-test of the failure path every tensor-core kernel relies on: a wait on
// an mbarrier that nothing will complete gives up after its limit, records
// the timeout in the status word and lets the kernel end, so the caller gets
// DPGB_ETIMEOUT and the CUDA context stays usable.
#include "common.cuh"
#include "tc.cuh"

namespace dpgb {
namespace {

__global__ void wait_selftest_kernel(int* __restrict__ status, unsigned long long limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);  // one arrival would complete phase 0: none comes
    tc::fence_mbar_init();
  }
  __syncthreads();
  const bool ok = tc::mbar_wait_for(&bar, 0, status + kStatusTimeout, limit_ns);
  if (ok && threadIdx.x == 0) status[kStatusOverflow] = 1;  // cannot happen: the wait had nothing to wait for
}

}  // namespace
}  // namespace dpgb

extern "C" int dpgb_selftest_wait_timeout(double limit_ms, void* stream) {
  using namespace dpgb;
  clear_error();
  if (!(limit_ms > 0.0 && limit_ms <= 1000.0)) return fail(DPGB_EINVAL, "limit_ms must be in (0, 1000]");
  cudaStream_t st = as_stream(stream);
  int* status = nullptr;
  DPGB_CUDA(cudaMalloc(&status, sizeof(int) * kStatusSlots));
  int h[kStatusSlots] = {};
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st);
  if (e == cudaSuccess) {
    wait_selftest_kernel<<<1, 32, 0, st>>>(status, (unsigned long long)(limit_ms * 1e6));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, status, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(status);
  if (e != cudaSuccess) return fail(DPGB_ECUDA, std::string("wait self-test: ") + cudaGetErrorString(e));
  if (h[kStatusOverflow]) return fail(DPGB_ECUDA, "wait self-test: an mbarrier completed with no arrival");
  if (h[kStatusTimeout]) return fail(DPGB_ETIMEOUT, "bounded mbarrier wait timed out (self-test)");
  return DPGB_OK;
}
