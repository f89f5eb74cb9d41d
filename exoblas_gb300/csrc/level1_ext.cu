// nrm2 and iamax: standard level-1 routines the reference does not have
// (README.md:15 -- Exo lacked the value-dependent control they need), with
// the reference BLAS semantics (the caller handles N < 1 and, for iamax,
// incX < 1): iamax returns the 0-based index (as cblas_i?amax) of the first
// element of largest magnitude, NaNs never win except a NaN in the first
// position (the sequential loop starts from |x[0]| and tests `>`).
//
// Both are one streaming pass with per-thread partials, a fixed-order warp
// and block combination and a last-arriving-CTA combination of the per-CTA
// partials in CTA order (deterministic).  nrm2 accumulates the squares in
// FP64: exact enough and overflow-free for FP32 inputs; for FP64 inputs
// whose largest magnitude lies outside [2^-490, 2^490] (the squares could
// overflow or underflow) a second pass rescales by a power of two, launched
// always and returning at once unless the first pass asked for it, so the
// call never waits on the host.
#include <cuda_runtime.h>

#include <climits>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace l1 {

namespace ext {

constexpr int kT = 256;

__device__ __forceinline__ double nan_max(double a, double b) { return (b > a || b != b) ? b : a; }

struct Part2 {
  double ss, mx;
};

__device__ __forceinline__ Part2 part2_reduce_block(Part2 v, Part2 *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.ss += __shfl_xor_sync(0xffffffffu, v.ss, o);
    v.mx = nan_max(v.mx, __shfl_xor_sync(0xffffffffu, v.mx, o));
  }
  if (lane == 0) sh[w] = v;
  __syncthreads();
  Part2 r{0.0, 0.0};
  if (threadIdx.x == 0)
    for (int i = 0; i < kT / 32; ++i) {
      r.ss += sh[i].ss;
      r.mx = nan_max(r.mx, sh[i].mx);
    }
  __syncthreads();
  return r;  // valid in thread 0
}

// pass 1: sum of squares and largest magnitude.  flag[0] receives the
// binary exponent to rescale by (0: not needed).
template <typename T>
__global__ void __launch_bounds__(kT) nrm2_kernel(long n, const T *__restrict__ x, long inc, Part2 *partials,
                                                  unsigned *counter, T *result, int *flag) {
  __shared__ Part2 sh[kT / 32];
  __shared__ bool last;
  Part2 acc{0.0, 0.0};
  for (long i = long(blockIdx.x) * kT + threadIdx.x; i < n; i += long(gridDim.x) * kT) {
    const double v = fabs(double(x[i * inc]));
    acc.ss = fma(v, v, acc.ss);
    acc.mx = nan_max(acc.mx, v);
  }
  Part2 tot = part2_reduce_block(acc, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = tot;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  Part2 g{0.0, 0.0};
  for (unsigned b = 0; b < gridDim.x; ++b) {
    const Part2 p = partials[b];
    g.ss += p.ss;
    g.mx = nan_max(g.mx, p.mx);
  }
  *counter = 0;
  int e = 0;
  if (sizeof(T) == 8 && g.mx == g.mx && g.mx != INFINITY && g.mx != 0.0 &&
      (g.mx > 0x1p490 || g.mx < 0x1p-490)) {
    e = ilogb(g.mx);
    if (e == 0) e = 1;  // 0 means "no rescale"
  }
  *flag = e;
  if (g.mx != g.mx)
    *result = T(g.mx);  // NaN
  else if (g.mx == INFINITY)
    *result = T(INFINITY);
  else
    *result = T(sqrt(g.ss));
}

// pass 2 (FP64 only, when pass 1 asked for it): sum of (x 2^-e)^2
template <typename T>
__global__ void __launch_bounds__(kT) nrm2_rescaled_kernel(long n, const T *__restrict__ x, long inc, Part2 *partials,
                                                           unsigned *counter, T *result, const int *flag) {
  __shared__ Part2 sh[kT / 32];
  __shared__ bool last;
  const int e = *flag;
  if (e == 0) return;
  Part2 acc{0.0, 0.0};
  for (long i = long(blockIdx.x) * kT + threadIdx.x; i < n; i += long(gridDim.x) * kT) {
    const double v = ldexp(fabs(double(x[i * inc])), -e);
    acc.ss = fma(v, v, acc.ss);
  }
  Part2 tot = part2_reduce_block(acc, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = tot;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double ss = 0.0;
  for (unsigned b = 0; b < gridDim.x; ++b) ss += partials[b].ss;
  *counter = 0;
  *const_cast<int *>(flag) = 0;  // every CTA has read it; the word returns to zero
  *result = T(ldexp(sqrt(ss), e));
}

template <typename T>
struct Best {
  T v;
  long i;
};

template <typename T>
__device__ __forceinline__ Best<T> better(Best<T> a, Best<T> b) {
  return (b.v > a.v || (b.v == a.v && b.i < a.i)) ? b : a;
}

template <typename T>
__global__ void __launch_bounds__(kT) iamax_kernel(long n, const T *__restrict__ x, long inc, Best<T> *partials,
                                                   unsigned *counter, size_t *result) {
  __shared__ Best<T> sh[kT / 32];
  __shared__ bool last;
  Best<T> acc{T(-1), LONG_MAX};
  for (long i = long(blockIdx.x) * kT + threadIdx.x; i < n; i += long(gridDim.x) * kT) {
    const T v = fabs(x[i * inc]);
    if (v > acc.v) acc = Best<T>{v, i};  // increasing i: the first of equal values stays
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Best<T> other{__shfl_xor_sync(0xffffffffu, acc.v, o), __shfl_xor_sync(0xffffffffu, acc.i, o)};
    acc = better(acc, other);
  }
  if (lane == 0) sh[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    Best<T> b = sh[0];
    for (int k = 1; k < kT / 32; ++k) b = better(b, sh[k]);
    partials[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  Best<T> g = partials[0];
  for (unsigned b = 1; b < gridDim.x; ++b) g = better(g, partials[b]);
  *counter = 0;
  const T x0 = x[0];
  *result = (x0 != x0 || g.i == LONG_MAX) ? size_t(0) : size_t(g.i);
}

inline long grid_for(long n) {
  long blocks = ceil_div(n, long(kT) * 4);
  if (blocks < 1) blocks = 1;
  if (blocks > grid_cap(4)) blocks = grid_cap(4);
  return blocks;
}

}  // namespace ext

template <typename T>
void nrm2(long n, const T *x, long incx, T *result) {
  using namespace ext;
  cudaStream_t s = ctx().stream;
  const long blocks = grid_for(n);
  Part2 *partials = static_cast<Part2 *>(scratch(sizeof(Part2) * size_t(blocks)));
  unsigned *counter = zero_words(2);
  int *flag = reinterpret_cast<int *>(counter + 1);
  nrm2_kernel<T><<<int(blocks), kT, 0, s>>>(n, x, incx, partials, counter, result, flag);
  count_launch();
  if (sizeof(T) == 8) {
    nrm2_rescaled_kernel<T><<<int(blocks), kT, 0, s>>>(n, x, incx, partials, counter, result, flag);
    count_launch();
  }
  EXB_LAUNCH("nrm2 kernel");
}

template <typename T>
void iamax(long n, const T *x, long incx, size_t *result) {
  using namespace ext;
  const long blocks = grid_for(n);
  Best<T> *partials = static_cast<Best<T> *>(scratch(sizeof(Best<T>) * size_t(blocks)));
  unsigned *counter = zero_words(1);
  iamax_kernel<T><<<int(blocks), kT, 0, ctx().stream>>>(n, x, incx, partials, counter, result);
  EXB_LAUNCH("iamax kernel");
  count_launch();
}

template void nrm2<float>(long, const float *, long, float *);
template void nrm2<double>(long, const double *, long, double *);
template void iamax<float>(long, const float *, long, size_t *);
template void iamax<double>(long, const double *, long, size_t *);

}  // namespace l1
}  // namespace exb
