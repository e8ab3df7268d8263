// prod_force_a without any device allocation.
//
// dpgb_prod_force_a_f64 obtains its scratch (per-pair forces, the sorted
// transpose of the neighbour list, a status word) from cudaMalloc on every
// call.  Some callers cannot do that: an MD engine that hands the library a
// device whose memory is owned by its own pool allocator (a cudaMalloc there
// fails or fragments the pool), or a tight MD inner loop where the implicit
// device-wide synchronisation of cudaMalloc / cudaFree would serialise work
// the application keeps in flight on other streams.  This variant keeps its
// scratch in one fixed array of this library's device image instead.
//
// Rules of the shared array:
//  * it is a file-scope __device__ array of kScratchBytes (11 MiB), present
//    on every GPU that loads the library until the process exits;
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it together
//    with the device's current CUDA context; a call that finds another
//    context there (the primary context was reset, or the caller made its
//    own) looks the address up again.  Make the first call on a device, and
//    the first after a context change, before any stream capture;
//  * every call reuses the same array and it keeps the last call's contents;
//    the call clears what must start at zero (counters, status) itself;
//  * two calls whose kernels overlap on the GPU (different streams, or
//    different host threads) race on the array: serialise them.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "nlist.cuh"

namespace dpgb {
namespace {

constexpr long long kMaxPairs = 262144;  // nframes * nloc * nnei
constexpr long long kMaxKeys = 262144;   // nframes * nall
// pair forces (3 doubles per pair) + keys + transpose (3*(keys+1) + pairs
// ints) + status, each region 256-byte aligned
constexpr size_t kPfBytes = ((size_t)kMaxPairs * 3 * sizeof(double) + 255) / 256 * 256;
constexpr size_t kKeyBytes = ((size_t)kMaxPairs * sizeof(int) + 255) / 256 * 256;
constexpr size_t kTrBytes = ((size_t)(3 * (kMaxKeys + 1) + kMaxPairs) * sizeof(int) + 256 + 255) / 256 * 256;
constexpr size_t kStatusBytes = 256;
constexpr size_t kScratchBytes = kPfBytes + kKeyBytes + kTrBytes + kStatusBytes;

static __device__ __align__(256) unsigned char g_prod_force_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};

// the calling thread's current CUDA context (the driver's cuCtxGetCurrent,
// taken through the runtime); null when unavailable
CUcontext current_context() {
  static PFN_cuCtxGetCurrent_v4000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
  }();
  CUcontext c = nullptr;
  if (fn && fn(&c) != CUDA_SUCCESS) c = nullptr;
  return c;
}

// device address of the scratch array on the current device: looked up once
// per device and context
int scratch_address(unsigned char** out) {
  int dev = 0;
  DPGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(DPGB_EINVAL, "device index beyond the supported range");
  const CUcontext ctx = current_context();  // null before the runtime made one current
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev] || !ctx || ctx != g_scratch_ctx[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_prod_force_scratch);
    if (e != cudaSuccess)
      return fail(DPGB_ECUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    g_scratch_ctx[dev] = current_context();  // the lookup made the device's context current
  }
  *out = g_scratch_ptr[dev];
  return DPGB_OK;
}

__global__ void pair_force_static_kernel(double* __restrict__ pf, const double* __restrict__ nd,
                                         const double* __restrict__ ed, long long npair) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  double f[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const double n = nd[4 * p + a];
#pragma unroll
    for (int k = 0; k < 3; ++k) f[k] += n * ed[(4 * p + a) * 3 + k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) pf[3 * p + k] = f[k];
}

__global__ void keys_static_kernel(int* __restrict__ keys, const int* __restrict__ nlist, long long npair,
                                   long long per_frame, int nall) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int j = nlist[p];
  keys[p] = (j < 0 || j >= nall) ? -1 : (int)(j + (p / per_frame) * nall);
}

__global__ void gather_static_kernel(double* __restrict__ force, const double* __restrict__ pf, Transpose tr,
                                     int nloc, int nall, int nnei, int nframes) {
  const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (long long)nframes * nall) return;
  const int f = (int)(q / nall), j = (int)(q % nall);
  double acc[3] = {0, 0, 0};
  if (j < nloc) {
    const double* row = pf + ((size_t)f * nloc + j) * nnei * 3;
    for (int s = 0; s < nnei; ++s)
#pragma unroll
      for (int k = 0; k < 3; ++k) acc[k] -= row[3 * s + k];
  }
  for (int t = tr.offsets[q]; t < tr.offsets[q + 1]; ++t) {
    const int p = tr.pairs[t];
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[k] += pf[3 * (size_t)p + k];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) force[3 * q + k] = acc[k];
}

}  // namespace
}  // namespace dpgb

using namespace dpgb;

extern "C" int dpgb_prod_force_a_f64_noalloc(double* force, const double* net_deriv, const double* env_deriv,
                                             const int* nlist, int nloc, int nall, int nnei, int nframes,
                                             void* stream) {
  clear_error();
  if (nloc < 0 || nall < nloc || nnei < 0 || nframes < 1)
    return fail(DPGB_EINVAL, "prod_force_a_noalloc: bad sizes");
  const long long npair = (long long)nframes * nloc * nnei;
  const long long nkeys = (long long)nframes * nall;
  if (npair > kMaxPairs || nkeys > kMaxKeys)
    return fail(DPGB_EINVAL, "prod_force_a_noalloc: nframes*nloc*nnei and nframes*nall must not exceed " +
                                 std::to_string(kMaxPairs) + " (got " + std::to_string(npair) + " and " +
                                 std::to_string(nkeys) + "); use dpgb_prod_force_a_f64 for larger systems");
  if (nkeys == 0) return DPGB_OK;
  unsigned char* base = nullptr;
  DPGB_TRY(scratch_address(&base));
  cudaStream_t st = as_stream(stream);
  double* pf = reinterpret_cast<double*>(base);
  int* keys = reinterpret_cast<int*>(base + kPfBytes);
  void* trw = base + kPfBytes + kKeyBytes;
  int* status = reinterpret_cast<int*>(base + kPfBytes + kKeyBytes + kTrBytes);
  // the array keeps the previous call's contents: clear the status word
  // (the transpose clears its own counters)
  DPGB_CUDA(cudaMemsetAsync(status, 0, sizeof(int) * kStatusSlots, st));
  if (npair > 0) {
    pair_force_static_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(pf, net_deriv, env_deriv, npair);
    DPGB_TRY(check_launch("pair_force_noalloc"));
    keys_static_kernel<<<ceil_div(npair, 256), 256, 0, st>>>(keys, nlist, npair, (long long)nloc * nnei, nall);
    DPGB_TRY(check_launch("keys_noalloc"));
  }
  Transpose tr;
  DPGB_TRY(launch_transpose(tr, keys, npair, (int)nkeys, 0, trw, status, st));
  gather_static_kernel<<<ceil_div(nkeys, 256), 256, 0, st>>>(force, pf, tr, nloc, nall, nnei, nframes);
  DPGB_TRY(check_launch("gather_noalloc"));
  int h[kStatusSlots];
  DPGB_TRY(read_status(status, st, h));
  if (h[kStatusOverflow] > 0)
    return fail(DPGB_EOVERFLOW, "prod_force_a_noalloc: an atom appears in more than 2048 rows");
  return DPGB_OK;
}
