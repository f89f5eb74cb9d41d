// Shared definitions for the exoblas_gb300 CUDA library (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>

#include "../../include/exoblas.h"

namespace exb {

// CBLAS flag values (reference: src/common/cblas_enums.py:4-33)
constexpr int kRowMajor = 101;
constexpr int kColMajor = 102;
constexpr int kNoTrans = 111;
constexpr int kTrans = 112;
constexpr int kConjTrans = 113;
constexpr int kUpper = 121;
constexpr int kLower = 122;
constexpr int kNonUnit = 131;
constexpr int kUnit = 132;
constexpr int kLeft = 141;
constexpr int kRight = 142;

// Thrown inside the library only; every exported entry point catches it and
// turns it into a status code (the C ABI never lets an exception escape).
struct Error {
  int status;
  const char *what;
};

[[noreturn]] void fail(int status, const char *what);
void check_cuda(cudaError_t e, const char *what);
#define EXB_CUDA(call) ::exb::check_cuda((call), #call)
#define EXB_LAUNCH(what) ::exb::check_cuda(cudaGetLastError(), what)

// A grow-only device buffer owned by one host thread and device.
struct Arena {
  void *ptr = nullptr;
  size_t bytes = 0;
  void *get(size_t need);  // may reallocate: never hold a pointer across get()
  void release();
};

// Per-thread, per-device state: the stream every call of this thread is
// issued on, the scratch used by multi-pass kernels and the staging buffers
// that hold copies of host operands.
struct Context {
  int device = 0;
  int sm_count = 0;
  bool pageable_direct = false;  // the device reads pageable host memory through the host page tables
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  bool blocking = true;
  int precision = EXOBLAS_PRECISION_NATIVE;
  bool status_pending = false;  // a kernel with bounded waits was queued
  // a second stream for work that runs beside the main stream's kernel (the
  // extra streaming CTAs of the clustered trsv), joined back through events
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  Arena scratch;      // partial sums, flags, counters (zeroed regions noted per kernel)
  Arena counters;     // small zero-initialised words; kernels leave them zero
  Arena staging[6];   // device copies of host operands, one slot per operand
  ~Context();
};

Context &ctx();

// Device scratch of at least `bytes` bytes (256-byte aligned) from the
// calling thread's arena.  Valid until the next scratch() call.
void *scratch(size_t bytes);
// `n` 32-bit words that are zero on entry and that kernels using them must
// leave zero on exit (reduction arrival counters).
unsigned int *zero_words(int n);

inline int grid_cap(int blocks_per_sm) { return ctx().sm_count * blocks_per_sm; }

__host__ __device__ inline long ceil_div(long a, long b) { return (a + b - 1) / b; }

// 16-byte vector of T
template <typename T>
struct V16;
template <>
struct V16<float> {
  using type = float4;
  static constexpr int N = 4;
};
template <>
struct V16<double> {
  using type = double2;
  static constexpr int N = 2;
};

template <typename T>
__device__ __forceinline__ T vget(const typename V16<T>::type &v, int i);
template <>
__device__ __forceinline__ float vget<float>(const float4 &v, int i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}
template <>
__device__ __forceinline__ double vget<double>(const double2 &v, int i) {
  return i == 0 ? v.x : v.y;
}
template <typename T>
__device__ __forceinline__ void vset(typename V16<T>::type &v, int i, T x);
template <>
__device__ __forceinline__ void vset<float>(float4 &v, int i, float x) {
  if (i == 0) v.x = x;
  else if (i == 1) v.y = x;
  else if (i == 2) v.z = x;
  else v.w = x;
}
template <>
__device__ __forceinline__ void vset<double>(double2 &v, int i, double x) {
  if (i == 0) v.x = x;
  else v.y = x;
}

// Streaming loads that do not allocate in L1 (data touched once).
template <typename V>
__device__ __forceinline__ V ld_stream(const V *p) {
  return __ldcs(p);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Fixed-order block sum (warp tree, then warp 0 over the per-warp results).
// Returns the total in thread 0.  `sh` needs blockDim.x / 32 entries.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T *sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  T r = 0;
  if (warp == 0) {
    r = lane < (int)(blockDim.x >> 5) ? sh[lane] : T(0);
    r = warp_sum(r);
  }
  return r;
}

// Alignment helpers
inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace exb
