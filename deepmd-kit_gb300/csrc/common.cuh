// Shared helpers of the dpgb CUDA library: error plumbing, launch checks and
// small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "dpgb.h"

namespace dpgb {

// Thread-local last-error text behind dpgb_last_error().
void set_error(const std::string& msg);
void clear_error();

inline int fail(int code, const std::string& msg) {
  set_error(msg);
  return code;
}

inline int check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    return fail(DPGB_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
  return DPGB_OK;
}

// After a launch: configuration errors surface here (asynchronous faults are
// reported by the next synchronising call).
inline int check_launch(const char* what) {
  return check_cuda(cudaGetLastError(), what);
}

#define DPGB_TRY(x)                 \
  do {                              \
    int _rc = (x);                  \
    if (_rc != DPGB_OK) return _rc; \
  } while (0)

#define DPGB_CUDA(x) DPGB_TRY(::dpgb::check_cuda((x), #x))

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// streaming multiprocessors of the current device (looked up once)
inline int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

// Device-side status word layout (one int per code, atomicMax'ed).
// kStatusNonFinite: 1 + the first input atom seen with a non-finite
// coordinate (any such atom; the others stay valid to read).
enum StatusSlot {
  kStatusOverflow = 0,
  kStatusOverflowAtom = 1,
  kStatusTimeout = 2,
  kStatusNonFinite = 6,
  kStatusSlots = 8
};

// a coordinate triple that is not finite (NaN or +-inf) flags the status
__device__ __forceinline__ void flag_nonfinite(const double* x, int atom, int* status) {
  if (status && !(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) atomicMax(status + kStatusNonFinite, atom + 1);
}

// Work items of a persistent kernel.  With a queue (an int zeroed before the
// launch) each CTA takes the next item index from it when it finishes one,
// so CTAs that drew short items take more of them; without a queue the
// items go to the CTAs in a fixed stride.  Every thread of the CTA calls
// these (they hold barriers); the item index is uniform over the CTA.
__device__ __forceinline__ int work_first(int* queue, int* slot) {
  if (threadIdx.x == 0) *slot = queue ? atomicAdd(queue, 1) : (int)blockIdx.x;
  __syncthreads();
  return *slot;
}
__device__ __forceinline__ int work_next(int* queue, int item, int* slot) {
  __syncthreads();  // every thread has read the current index
  if (threadIdx.x == 0) *slot = queue ? atomicAdd(queue, 1) : item + (int)gridDim.x;
  __syncthreads();
  return *slot;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Exact sum of two floats as s + e (Knuth's two-sum; needs IEEE order of
// operations, which holds without fast-math).  Sums of FP32 terms kept as
// hi + lo this way are as accurate as FP64 accumulation and use the FP32
// pipe, not the (narrow) FP64 one.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
// (a + s) - b in FP32 from hi + lo splits of each term: two error-free sums
// (two_sum) carry the rounding of the high parts into the low-order part,
// so the result is the exact value rounded once more, within 2^-24 of it
// plus a term of order 2^-48 of the operands (FP32 instructions only; the
// FP64 pipe is narrow on this part)
__device__ __forceinline__ float disp_split(float ah, float al, float sh, float sl, float bh, float bl) {
  float s1, e1, s2, e2;
  two_sum(ah, sh, s1, e1);
  two_sum(s1, -bh, s2, e2);
  return s2 + (((al + sl) - bl) + (e1 + e2));
}
__device__ __forceinline__ void comp_add(float& hi, float& lo, float x) {
  float e;
  two_sum(hi, x, hi, e);
  lo += e;
}
// warp-wide compensated sum (xor tree: the same value in every lane)
__device__ __forceinline__ double warp_comp_sum(float hi, float lo) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, hi, o), ol = __shfl_xor_sync(0xffffffffu, lo, o);
    float e;
    two_sum(hi, oh, hi, e);
    lo += ol + e;
  }
  return (double)hi + (double)lo;
}

// Division of non-negative 31-bit integers by a divisor d >= 1 fixed for a
// launch, by one widening multiply and a shift (Granlund and Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994): with
// 2^l >= d and m = ceil(2^(31+l) / d) < 2^32, floor(n m / 2^(31+l)) = n / d
// for every 0 <= n < 2^31 (the error m d - 2^(31+l) < d adds less than 1/d).
// scale of the 2^-32 fixed-point force sums (64-bit integers)
constexpr float kFixScale = 4294967296.f;  // 2^32

struct FastDiv {
  unsigned m = 1u << 31;
  int s = 31;
  FastDiv() = default;
  explicit FastDiv(int d) {
    int l = 0;
    while ((1LL << l) < d) ++l;
    s = 31 + l;
    m = (unsigned)(((1ULL << s) + (unsigned long long)d - 1) / (unsigned long long)d);
  }
  __host__ __device__ __forceinline__ int div(int n) const {
    return (int)(((unsigned long long)(unsigned)n * m) >> s);
  }
};

// Scoped device allocation used by op-level entry points (workspace).
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer&) = delete;
  DeviceBuffer& operator=(const DeviceBuffer&) = delete;
  ~DeviceBuffer() {
    if (ptr) cudaFree(ptr);
  }
  int alloc(size_t n) {
    if (n <= bytes) return DPGB_OK;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    if (n == 0) return DPGB_OK;
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e != cudaSuccess) {
      ptr = nullptr;
      return fail(DPGB_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    bytes = n;
    return DPGB_OK;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(ptr);
  }
};

// Device scratch reused across the calls of one host thread (grow-only,
// one buffer per slot, reallocated when the thread's current device
// changes): a call that uses it must be done with it on the device before
// it returns (the op-level entries that use it synchronise their stream
// before returning), so the thread's next call may overwrite it.
inline DeviceBuffer& thread_scratch(int slot) {
  struct Slot {
    DeviceBuffer buf;
    int device = -1;
  };
  thread_local Slot slots[4];
  Slot& s = slots[slot & 3];
  int dev = 0;
  cudaGetDevice(&dev);
  if (s.device != dev) {
    if (s.buf.ptr) cudaFree(s.buf.ptr);
    s.buf.ptr = nullptr;
    s.buf.bytes = 0;
    s.device = dev;
  }
  return s.buf;
}

// Page-locked host staging (copies to and from it run asynchronously and at
// full link speed; the caller's own arrays are pageable).
struct PinnedBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  PinnedBuffer() = default;
  PinnedBuffer(const PinnedBuffer&) = delete;
  PinnedBuffer& operator=(const PinnedBuffer&) = delete;
  ~PinnedBuffer() {
    if (ptr) cudaFreeHost(ptr);
  }
  int alloc(size_t n) {
    if (n <= bytes) return DPGB_OK;
    if (ptr) cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
    if (n == 0) return DPGB_OK;
    cudaError_t e = cudaHostAlloc(&ptr, n, cudaHostAllocDefault);
    if (e != cudaSuccess) {
      ptr = nullptr;
      return fail(DPGB_ENOMEM, std::string("cudaHostAlloc: ") + cudaGetErrorString(e));
    }
    bytes = n;
    return DPGB_OK;
  }
  template <typename T>
  T* as() const {
    return reinterpret_cast<T*>(ptr);
  }
};

}  // namespace dpgb
