// dasum on integer significand sums (below), and nrm2 and iamax:
// standard level-1 routines the reference does not have
// (README.md:15 -- Exo lacked the value-dependent control they need), with
// the reference BLAS semantics (the caller handles N < 1 and, for iamax,
// incX < 1): iamax returns the 0-based index (as cblas_i?amax) of the first
// element of largest magnitude, NaNs never win except a NaN in the first
// position (the sequential loop starts from |x[0]| and tests `>`).
//
// Both are one streaming pass (16-byte vector loads for unit stride) with
// per-thread partials, a fixed-order warp and block combination and a
// last-arriving-CTA combination of the per-CTA partials in CTA order
// (deterministic).  Per element they do little floating-point work -- this
// GPU's FP64 pipe is far slower than HBM: magnitudes are compared as
// integer bit patterns, and FP32 squares are accumulated exactly as FP32
// pairs (product error through fma, TwoSum), FP64 squares with one FMA.
// When the largest magnitude lies outside [2^-40, 2^40] (FP32) or
// [2^-490, 2^490] (FP64), where sums of squares could overflow or lose the
// small terms to underflow, a
// second pass rescales by a power of two; it is launched always and returns
// at once unless the first pass asked for it, so the call never waits on
// the host.
#include <cuda_runtime.h>

#include <climits>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace l1 {

namespace ext {

constexpr int kT = 256;
constexpr int kU = 4;  // vectors in flight per thread

// magnitude keys: |x| as an unsigned bit pattern orders like |x| for every
// non-NaN value, and every NaN's key is above the infinity's
template <typename T>
struct Key;
template <>
struct Key<float> {
  using U = unsigned;
  static constexpr U kInf = 0x7f800000u;
  static __device__ __forceinline__ U of(float x) { return __float_as_uint(x) & 0x7fffffffu; }
  static __device__ __forceinline__ double value(U k) { return double(__uint_as_float(k)); }
};
template <>
struct Key<double> {
  using U = unsigned long long;
  static constexpr U kInf = 0x7ff0000000000000ull;
  static __device__ __forceinline__ U of(double x) { return U(__double_as_longlong(x)) & 0x7fffffffffffffffull; }
  static __device__ __forceinline__ double value(U k) { return __longlong_as_double((long long)k); }
};

// 32-bit magnitude keys for nrm2's range check: the FP32 key itself; for
// FP64 the high word of |x| with bit 0 set when the low word is nonzero, so
// a NaN whose payload lies in the low word still sorts above the infinity.
// Keys order like the magnitudes up to the low word, which the range check
// does not need.  (A 64-bit key max per element doubled dnrm2's FP64-pipe
// time on GB300.)
template <typename T>
struct Mag32;
template <>
struct Mag32<float> {
  static __device__ __forceinline__ unsigned of(float x) { return Key<float>::of(x); }
  static __device__ __forceinline__ double value(unsigned k) { return Key<float>::value(k); }
};
template <>
struct Mag32<double> {
  static __device__ __forceinline__ unsigned of(double x) {
    return (unsigned(__double2hiint(x)) & 0x7fffffffu) | unsigned(__double2loint(x) != 0);
  }
  static __device__ __forceinline__ double value(unsigned k) { return __hiloint2double(int(k), 0); }
};

// sum of squares: FP32 inputs through exact products p + e (e = fma(x, x, -p))
// accumulated with TwoSum in an FP32 pair (no FP64 work per element); FP64
// inputs with one FP64 FMA per element.  The largest magnitude is kept as
// an integer key (no floating-point work).
template <typename T>
struct SumSq;
template <>
struct SumSq<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float p = x * x;
    const float e = fmaf(x, x, -p);
    const float s = hi + p;
    const float z = s - hi;
    lo += ((hi - (s - z)) + (p - z)) + e;
    hi = s;
  }
  __device__ __forceinline__ double get() const { return double(hi) + double(lo); }
};
template <>
struct SumSq<double> {
  double ss = 0.0;
  __device__ __forceinline__ void add(double x) { ss = fma(x, x, ss); }
  __device__ __forceinline__ double get() const { return ss; }
};

// A per-CTA partial of nrm2: the sum of squares and the largest magnitude
// as its 32-bit key (integer max all the way: NaN keys sort above the
// infinity's, so a NaN anywhere survives the combination).
struct Part2 {
  double ss;
  unsigned mk;
};

// FP32 pairs (hi + lo) added with TwoSum: the FP32 path combines its slots
// and lanes this way and converts to FP64 once per warp.  (Per-thread FP64
// conversions and adds at the end of the stream kept GB300's slow FP64 pipe
// 19% busy in snrm2.)
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const float s = a.hi + b.hi;
  const float z = s - a.hi;
  const float e = ((a.hi - (s - z)) + (b.hi - z)) + (a.lo + b.lo);
  const float hi = s + e;
  return F2{hi, e - (hi - s)};
}

// Block combination in a fixed order: the warp tree, then thread 0 over
// the warps.  Returns the total in thread 0.
__device__ __forceinline__ Part2 part2_block(double ss, unsigned mk, Part2 *sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ss += __shfl_xor_sync(0xffffffffu, ss, o);
    mk = max(mk, __shfl_xor_sync(0xffffffffu, mk, o));
  }
  if (lane == 0) sh[w] = Part2{ss, mk};
  __syncthreads();
  Part2 r{0.0, 0u};
  if (threadIdx.x == 0)
    for (int i = 0; i < kT / 32; ++i) {
      r.ss += sh[i].ss;
      r.mk = max(r.mk, sh[i].mk);
    }
  __syncthreads();
  return r;
}

// The per-thread slots of a streaming pass, combined over the block.
template <typename T>
__device__ __forceinline__ Part2 sumsq_block(const SumSq<T> (&acc)[kU], unsigned mk, Part2 *sh) {
  if constexpr (sizeof(T) == 4) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    F2 t{acc[0].hi, acc[0].lo};
#pragma unroll
    for (int u = 1; u < kU; ++u) t = f2_add(t, F2{acc[u].hi, acc[u].lo});
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const F2 other{__shfl_xor_sync(0xffffffffu, t.hi, o), __shfl_xor_sync(0xffffffffu, t.lo, o)};
      t = f2_add(t, other);
      mk = max(mk, __shfl_xor_sync(0xffffffffu, mk, o));
    }
    if (lane == 0) sh[w] = Part2{double(t.hi) + double(t.lo), mk};
    __syncthreads();
    Part2 r{0.0, 0u};
    if (threadIdx.x == 0)
      for (int i = 0; i < kT / 32; ++i) {
        r.ss += sh[i].ss;
        r.mk = max(r.mk, sh[i].mk);
      }
    __syncthreads();
    return r;
  } else {
    double ss = 0.0;
#pragma unroll
    for (int u = 0; u < kU; ++u) ss += acc[u].get();
    return part2_block(ss, mk, sh);
  }
}

// The vector loop of for_each with index type I: 32-bit when the vector
// count allows it, 64-bit otherwise.
template <typename I, typename T, class F>
__device__ __forceinline__ void for_each_vec(I nvec, const typename V16<T>::type *__restrict__ xv, I gt, I stride,
                                             F &f) {
  using V = typename V16<T>::type;
  constexpr int VN = V16<T>::N;
  I v = gt;
  // the next kU vectors are loaded before the current ones are consumed
  V a[kU], b[kU];
  bool have = v + (kU - 1) * stride < nvec;
  if (have) {
#pragma unroll
    for (int u = 0; u < kU; ++u) a[u] = ld_stream(xv + v + u * stride);
  }
  while (have) {
    const I vn = v + kU * stride;
    const bool more = vn + (kU - 1) * stride < nvec;
    if (more) {
#pragma unroll
      for (int u = 0; u < kU; ++u) b[u] = ld_stream(xv + vn + u * stride);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u)
#pragma unroll
      for (int e = 0; e < VN; ++e) f(u, vget<T>(a[u], e), long(v + u * stride) * VN + e);
#pragma unroll
    for (int u = 0; u < kU; ++u) a[u] = b[u];
    v = vn;
    have = more;
  }
  for (; v < nvec; v += stride) {
    const V c = ld_stream(xv + v);
#pragma unroll
    for (int e = 0; e < VN; ++e) f(0, vget<T>(c, e), long(v) * VN + e);
  }
}

// FP64 data as 32-bit words: calls f(slot, hi, lo, index) for each element
// (hi and lo the words of its bit pattern), with the pipelined loop of
// for_each_vec over 16-byte vectors of two elements.  The buffers hold no
// FP64 values: with double2 buffers idamax kept GB300's FP64 pipe 72% busy
// without a single FP64 arithmetic instruction; with these it is idle.
template <typename I, class F>
__device__ __forceinline__ void for_each_words(I nvec, const uint4 *__restrict__ xv, I gt, I stride, F &f) {
  I v = gt;
  uint4 a[kU], b[kU];
  bool have = v + (kU - 1) * stride < nvec;
  if (have) {
#pragma unroll
    for (int u = 0; u < kU; ++u) a[u] = ld_stream(xv + v + u * stride);
  }
  while (have) {
    const I vn = v + kU * stride;
    const bool more = vn + (kU - 1) * stride < nvec;
    if (more) {
#pragma unroll
      for (int u = 0; u < kU; ++u) b[u] = ld_stream(xv + vn + u * stride);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      f(u, a[u].y, a[u].x, long(v + u * stride) * 2);
      f(u, a[u].w, a[u].z, long(v + u * stride) * 2 + 1);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) a[u] = b[u];
    v = vn;
    have = more;
  }
  for (; v < nvec; v += stride) {
    const uint4 c = ld_stream(xv + v);
    f(0, c.y, c.x, long(v) * 2);
    f(0, c.w, c.z, long(v) * 2 + 1);
  }
}

// for_each for FP64 data as words: f(slot, hi, lo, index)
template <class F>
__device__ __forceinline__ void words(long n, const double *__restrict__ x, long inc, bool vec, F &f) {
  const long stride = long(gridDim.x) * kT, gt = long(blockIdx.x) * kT + threadIdx.x;
  auto one = [&](double d, long i) { f(0, unsigned(__double2hiint(d)), unsigned(__double2loint(d)), i); };
  if (vec) {
    const long nvec = n / 2;
    const uint4 *xv = reinterpret_cast<const uint4 *>(x);
    if (nvec + 2 * kU * stride < (1L << 32))
      for_each_words<unsigned>(unsigned(nvec), xv, unsigned(gt), unsigned(stride), f);
    else
      for_each_words<long>(nvec, xv, gt, stride, f);
    for (long i = nvec * 2 + gt; i < n; i += stride) one(x[i], i);
  } else {
    for (long i = gt; i < n; i += stride) one(x[i * inc], i);
  }
}

// Calls f(slot, value, index) for this thread's elements: 16-byte vectors
// when x is unit-stride and aligned, kU of them consumed per step while the
// next kU are in flight; slot u < kU names an independent accumulator (the
// elements of one slot come in increasing index order).
template <typename T, class F>
__device__ __forceinline__ void for_each(long n, const T *__restrict__ x, long inc, bool vec, F &&f) {
  using V = typename V16<T>::type;
  constexpr int VN = V16<T>::N;
  const long stride = long(gridDim.x) * kT;
  const long gt = long(blockIdx.x) * kT + threadIdx.x;
  if (vec) {
    const long nvec = n / VN;
    const V *xv = reinterpret_cast<const V *>(x);
    // 32-bit indices while every index the loop forms (up to nvec plus
    // 2 kU strides) stays below 2^32
    if (nvec + 2 * kU * stride < (1L << 32))
      for_each_vec<unsigned, T>(unsigned(nvec), xv, unsigned(gt), unsigned(stride), f);
    else
      for_each_vec<long, T>(nvec, xv, gt, stride, f);
    for (long i = nvec * VN + gt; i < n; i += stride) f(0, x[i], i);
  } else {
    for (long i = gt; i < n; i += stride) f(0, x[i * inc], i);
  }
}

// pass 1: sum of squares and largest magnitude.  flag[0] receives the
// binary exponent to rescale by (0: not needed).
template <typename T>
__global__ void __launch_bounds__(kT) nrm2_kernel(long n, const T *__restrict__ x, long inc, bool vec,
                                                  Part2 *partials, unsigned *counter, T *result, int *flag) {
  using K = Mag32<T>;
  __shared__ Part2 sh[kT / 32];
  __shared__ bool last;
  SumSq<T> acc[kU];
  unsigned mk = 0;
  for_each(n, x, inc, vec, [&](int u, T v, long) {
    acc[u].add(v);
    mk = max(mk, K::of(v));
  });
  Part2 tot = sumsq_block<T>(acc, mk, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = tot;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last CTA combines the per-CTA partials: thread t takes CTAs t,
  // t + kT, ... in order, then the fixed block tree
  double ss = 0.0;
  unsigned m = 0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kT) {
    ss += __ldcg(&partials[b].ss);
    m = max(m, __ldcg(&partials[b].mk));
  }
  const Part2 g = part2_block(ss, m, sh);
  if (threadIdx.x != 0) return;
  *counter = 0;
  const double mx = K::value(g.mk);
  // squares and per-thread sums of up to 2^20 of them stay in range and
  // normal while the largest magnitude lies in [tiny, lim]
  const double lim = sizeof(T) == 8 ? 0x1p490 : 0x1p40, tiny = sizeof(T) == 8 ? 0x1p-490 : 0x1p-40;
  int e = 0;
  if (mx == mx && mx != INFINITY && mx != 0.0 && (mx > lim || mx < tiny)) {
    e = ilogb(mx);
    if (e == 0) e = 1;  // 0 means "no rescale"
  }
  *flag = e;
  if (mx != mx)
    *result = T(mx);  // NaN
  else if (mx == INFINITY)
    *result = T(INFINITY);
  else
    *result = T(sqrt(g.ss));
}

// pass 2 (when pass 1 asked for it): sum of (x 2^-e)^2
template <typename T>
__global__ void __launch_bounds__(kT) nrm2_rescaled_kernel(long n, const T *__restrict__ x, long inc, bool vec,
                                                           Part2 *partials, unsigned *counter, T *result,
                                                           const int *flag) {
  __shared__ Part2 sh[kT / 32];
  __shared__ bool last;
  const int e = *flag;
  if (e == 0) return;
  const T sc = T(ldexp(1.0, -e));  // exact power of two
  SumSq<T> acc[kU];
  for_each(n, x, inc, vec, [&](int u, T v, long) { acc[u].add(v * sc); });
  Part2 tot = sumsq_block<T>(acc, 0u, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = tot;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double part = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kT) part += __ldcg(&partials[b].ss);
  const double ss = part2_block(part, 0u, sh).ss;
  if (threadIdx.x != 0) return;
  *counter = 0;
  *const_cast<int *>(flag) = 0;  // every CTA has read it; the word returns to zero
  *result = T(ldexp(sqrt(ss), e));
}

template <typename U>
struct Best {
  U k;  // magnitude key (0 before any element: no non-NaN key is below it... see better())
  long i;
};

// larger magnitude wins; equal magnitudes: the smaller index
template <typename U>
__device__ __forceinline__ Best<U> better(Best<U> a, Best<U> b) {
  return (b.k > a.k || (b.k == a.k && b.i < a.i)) ? b : a;
}

template <typename T>
__global__ void __launch_bounds__(kT) iamax_kernel(long n, const T *__restrict__ x, long inc, bool vec,
                                                   Best<typename Key<T>::U> *partials, unsigned *counter,
                                                   size_t *result) {
  using K = Key<T>;
  using U = typename K::U;
  __shared__ Best<U> sh[kT / 32];
  __shared__ bool last;
  // keys are stored + 1 so that 0 means "none yet"; NaN keys never enter
  Best<U> accs[kU];
  unsigned acc_hi[kU];  // FP64: high word of the slot's best magnitude
#pragma unroll
  for (int u = 0; u < kU; ++u) {
    accs[u] = Best<U>{0, LONG_MAX};
    acc_hi[u] = 0;
  }
  if constexpr (sizeof(T) == 8) {
    // FP64: the elements as 32-bit words; a test on the high word first (a
    // larger key needs a high word at least the best's), the 64-bit key only
    // then
    auto upd = [&](int u, unsigned hi, unsigned lo, long i) {
      const unsigned hk = hi & 0x7fffffffu;
      if (hk < acc_hi[u]) return;
      const U k = ((U(hk) << 32) | lo) + 1;
      if (k <= K::kInf + 1 && k > accs[u].k) {  // per slot increasing i: the first stays
        accs[u] = Best<U>{k, i};
        acc_hi[u] = hk;
      }
    };
    words(n, x, inc, vec, upd);
  } else {
    for_each(n, x, inc, vec, [&](int u, T v, long i) {
      const U k = K::of(v) + 1;
      if (k <= K::kInf + 1 && k > accs[u].k) accs[u] = Best<U>{k, i};  // per slot increasing i: the first stays
    });
  }
  Best<U> acc = accs[0];
#pragma unroll
  for (int u = 1; u < kU; ++u) acc = better(acc, accs[u]);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Best<U> other{__shfl_xor_sync(0xffffffffu, acc.k, o), __shfl_xor_sync(0xffffffffu, acc.i, o)};
    acc = better(acc, other);
  }
  if (lane == 0) sh[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    Best<U> b = sh[0];
    for (int q = 1; q < kT / 32; ++q) b = better(b, sh[q]);
    partials[blockIdx.x] = b;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last CTA: thread t combines CTAs t, t + kT, ..., then warp and
  // block trees (`better` is order-independent: larger key, then smaller index)
  Best<U> g{0, LONG_MAX};
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kT)
    g = better(g, Best<U>{__ldcg(&partials[b].k), __ldcg(&partials[b].i)});
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    Best<U> other{__shfl_xor_sync(0xffffffffu, g.k, o), __shfl_xor_sync(0xffffffffu, g.i, o)};
    g = better(g, other);
  }
  __syncthreads();  // sh is reused
  if (lane == 0) sh[w] = g;
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int q = 0; q < kT / 32; ++q) g = better(g, sh[q]);
  *counter = 0;
  const T x0 = x[0];
  *result = (x0 != x0 || g.i == LONG_MAX) ? size_t(0) : size_t(g.i);
}

// dasum (src/level1/asum.py:11-18) with a quarter of the FP64 work: one
// DADD per element (33.5 M warp lanes at n = 2^25) takes longer on GB300's
// FP64 unit than reading x from HBM, and the integer path alone keeps the
// integer ALU 77% busy (ncu; it also occupies the FP64 unit a third of the
// time), so one element in four takes an FP64 add and the others the
// integer path.  There |x| is taken apart from its bit pattern
// (the two 32-bit words that for_each_words hands over, so no FP64 value is
// held in a register) into its 53-bit significand and biased exponent e, and
// the significands accumulate in an unsigned 64-bit sum whose least
// significant bit weighs 2^(E - 1075), E the largest exponent this thread
// has seen.  A larger exponent shifts the sum down; a sum reaching 2^62 is
// halved (E + 1) before it could overflow.  Each element or shift truncates
// less than one unit of the final LSB, which weighs at most 2^-52 max|x|,
// so the error stays below 2 n eps sum|x|.  Infinities and NaNs go to an
// FP64 side sum so the IEEE result is kept; the per-thread parts and the
// block and grid combinations are FP64, in a fixed order.
struct AsumBits {
  unsigned long long acc = 0;
  int E = 1;
  double special = 0.0;
  // E stays <= 2046, so an infinity or NaN (e = 2047) always takes the rare
  // e > E branch; a sum that would need E = 2047 is beyond the FP64 range,
  // recorded as +inf in the side sum.
  __device__ __forceinline__ void add(unsigned hi, unsigned lo) {
    const unsigned h = hi & 0x7fffffffu;
    int e = int(h >> 20);
    const unsigned long long m =
        (static_cast<unsigned long long>((h & 0xfffffu) | (e ? 0x100000u : 0u)) << 32) | lo;
    e = max(e, 1);  // subnormals: significand without the hidden bit, exponent 1
    if (e > E) {
      if (e == 2047) {
        special += __hiloint2double(int(h), int(lo));
        return;
      }
      acc >>= min(e - E, 63);  // acc < 2^62: a shift by 63 leaves 0
      E = e;
    }
    acc += m >> min(E - e, 63);  // m < 2^53
    if (acc >> 62) {
      acc >>= 1;
      if (E < 2046)
        ++E;
      else
        special = __longlong_as_double(0x7ff0000000000000ll);
    }
  }
  __device__ __forceinline__ double part() const { return ldexp(double(acc), E - 1075) + special; }
};

__global__ void __launch_bounds__(kT) dasum_kernel(long n, const double *__restrict__ x, long inc, bool vec,
                                                   double *partials, unsigned *counter, double *result) {
  __shared__ Part2 sh[kT / 32];
  __shared__ bool last;
  // one element in four (the second of the vectors in slots 2 and 3 of the
  // unrolled loop: known at compile time, so no warp diverges) as one FP64
  // add, the others on the integer path, so both units share the work
  AsumBits acc;
  double sd = 0.0;
  auto f = [&](int u, unsigned hi, unsigned lo, long i) {
    if ((u & 2) && (i & 1))
      sd += fabs(__hiloint2double(int(hi), int(lo)));
    else
      acc.add(hi, lo);
  };
  words(n, x, inc, vec, f);
  const Part2 tot = part2_block(acc.part() + sd, 0u, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = tot.ss;
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the last CTA combines the per-CTA partials in CTA order
  double s = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += kT) s += __ldcg(partials + b);
  const double g = part2_block(s, 0u, sh).ss;
  if (threadIdx.x != 0) return;
  *counter = 0;
  *result = g;
}

inline long grid_for(long n, const void *kernel) {
  long blocks = ceil_div(n, long(kT) * 16);
  if (blocks < 1) blocks = 1;
  const int per_sm = resident_per_sm(kernel, kT);
  if (blocks > grid_cap(per_sm)) blocks = grid_cap(per_sm);
  return blocks;
}

}  // namespace ext

template <typename T>
void nrm2(long n, const T *x, long incx, T *result) {
  using namespace ext;
  cudaStream_t s = ctx().stream;
  const long blocks = grid_for(n, reinterpret_cast<const void *>(nrm2_kernel<T>));
  const bool vec = incx == 1 && aligned16(x);
  Part2 *partials = static_cast<Part2 *>(scratch(sizeof(Part2) * size_t(blocks)));
  unsigned *counter = zero_words(2);
  int *flag = reinterpret_cast<int *>(counter + 1);
  nrm2_kernel<T><<<int(blocks), kT, 0, s>>>(n, x, incx, vec, partials, counter, result, flag);
  nrm2_rescaled_kernel<T><<<int(blocks), kT, 0, s>>>(n, x, incx, vec, partials, counter, result, flag);
  EXB_LAUNCH("nrm2 kernel");
  count_launch(2);
}

template <typename T>
void iamax(long n, const T *x, long incx, size_t *result) {
  using namespace ext;
  using U = typename Key<T>::U;
  const long blocks = grid_for(n, reinterpret_cast<const void *>(iamax_kernel<T>));
  const bool vec = incx == 1 && aligned16(x);
  Best<U> *partials = static_cast<Best<U> *>(scratch(sizeof(Best<U>) * size_t(blocks)));
  unsigned *counter = zero_words(1);
  iamax_kernel<T><<<int(blocks), kT, 0, ctx().stream>>>(n, x, incx, vec, partials, counter, result);
  EXB_LAUNCH("iamax kernel");
  count_launch();
}

void dasum_words(long n, const double *x, long incx, double *result) {
  using namespace ext;
  if (n < 0) n = 0;
  const long blocks = grid_for(n, reinterpret_cast<const void *>(dasum_kernel));
  const bool vec = incx == 1 && aligned16(x);
  double *partials = static_cast<double *>(scratch(sizeof(double) * size_t(blocks)));
  unsigned *counter = zero_words(1);
  dasum_kernel<<<int(blocks), kT, 0, ctx().stream>>>(n, x, incx, vec, partials, counter, result);
  EXB_LAUNCH("dasum kernel");
  count_launch();
}

template void nrm2<float>(long, const float *, long, float *);
template void nrm2<double>(long, const double *, long, double *);
template void iamax<float>(long, const float *, long, size_t *);
template void iamax<double>(long, const double *, long, size_t *);

}  // namespace l1
}  // namespace exb
