// Level-1 kernels: 128-bit vectorised grid-stride element maps and
// deterministic two-pass reductions (warp shuffle tree, fixed-order block
// tree, then the last block to finish sums the per-block partials in block
// order).  Reference algorithms: src/level1/{asum,axpy,dot,dsdot,exo_copy,
// rot,rotm,scal,swap}.py.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace l1 {

constexpr int kThreads = 256;
constexpr int kUnroll = 4;

// ------------------------------------------------------------ element ops --
// Each op names which of x / y it reads and writes so that the kernels move
// only the bytes the reference loop moves.

template <typename T>
struct AxpyOp {  // axpy.py:9-12
  T a;
  static constexpr bool RX = true, RY = true, WX = false, WY = true;
  __device__ void operator()(T &x, T &y) const { y += a * x; }
};
template <typename T>
struct Axpy1Op {  // axpy.py:15-18
  static constexpr bool RX = true, RY = true, WX = false, WY = true;
  __device__ void operator()(T &x, T &y) const { y += x; }
};
template <typename T>
struct CopyOp {  // exo_copy.py:9-12
  static constexpr bool RX = true, RY = false, WX = false, WY = true;
  __device__ void operator()(T &x, T &y) const { y = x; }
};
template <typename T>
struct SwapOp {  // swap.py:9-15
  static constexpr bool RX = true, RY = true, WX = true, WY = true;
  __device__ void operator()(T &x, T &y) const {
    T t = x;
    x = y;
    y = t;
  }
};
template <typename T>
struct ScalOp {  // scal.py:9-12
  T a;
  static constexpr bool RX = true, RY = false, WX = true, WY = false;
  __device__ void operator()(T &x, T &) const { x = a * x; }
};
template <typename T>
struct ScalZeroOp {  // scal.py:15-19: writes 0.0 without reading x
  static constexpr bool RX = false, RY = false, WX = true, WY = false;
  __device__ void operator()(T &x, T &) const { x = T(0); }
};
template <typename T>
struct RotOp {  // rot.py:9-15
  T c, s;
  static constexpr bool RX = true, RY = true, WX = true, WY = true;
  __device__ void operator()(T &x, T &y) const {
    T xr = x;
    x = c * xr + s * y;
    y = -s * xr + c * y;
  }
};
template <typename T>
struct RotmNegOneOp {  // rotm.py:9-15
  T h00, h01, h10, h11;
  static constexpr bool RX = true, RY = true, WX = true, WY = true;
  __device__ void operator()(T &x, T &y) const {
    T xr = x;
    x = h00 * xr + h01 * y;
    y = h10 * xr + h11 * y;
  }
};
template <typename T>
struct RotmZeroOp {  // rotm.py:18-24
  T h01, h10;
  static constexpr bool RX = true, RY = true, WX = true, WY = true;
  __device__ void operator()(T &x, T &y) const {
    T xr = x;
    x = xr + h01 * y;
    y = h10 * xr + y;
  }
};
template <typename T>
struct RotmOneOp {  // rotm.py:27-33
  T h00, h11;
  static constexpr bool RX = true, RY = true, WX = true, WY = true;
  __device__ void operator()(T &x, T &y) const {
    T xr = x;
    x = h00 * xr + y;
    y = -xr + h11 * y;
  }
};

// Unit-stride map.  Elements [0, head) and [tail, n) are done one by one by
// block 0; [head, tail) is done in 16-byte vectors (x + head and y + head
// are 16-byte aligned).
template <typename T, class Op>
__global__ void __launch_bounds__(kThreads) map_unit(long n, T *__restrict__ x, T *__restrict__ y, Op op, int head) {
  using V = typename V16<T>::type;
  constexpr int VN = V16<T>::N;
  const long nvec = (n - head) / VN;
  const long tail = head + nvec * VN;
  V *xv = reinterpret_cast<V *>(x + head);
  V *yv = reinterpret_cast<V *>(y + head);
  const long stride = long(gridDim.x) * kThreads;
  long v = long(blockIdx.x) * kThreads + threadIdx.x;
  for (; v + (kUnroll - 1) * stride < nvec; v += kUnroll * stride) {
    V a[kUnroll], b[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      if (Op::RX) a[u] = ld_stream(xv + v + u * stride);
      if (Op::RY) b[u] = ld_stream(yv + v + u * stride);
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
#pragma unroll
      for (int e = 0; e < VN; ++e) {
        T xe = Op::RX ? vget<T>(a[u], e) : T(0);
        T ye = Op::RY ? vget<T>(b[u], e) : T(0);
        op(xe, ye);
        if (Op::WX) vset<T>(a[u], e, xe);
        if (Op::WY) vset<T>(b[u], e, ye);
      }
      if (Op::WX) __stcs(xv + v + u * stride, a[u]);
      if (Op::WY) __stcs(yv + v + u * stride, b[u]);
    }
  }
  for (; v < nvec; v += stride) {
    V a, b;
    if (Op::RX) a = ld_stream(xv + v);
    if (Op::RY) b = ld_stream(yv + v);
#pragma unroll
    for (int e = 0; e < VN; ++e) {
      T xe = Op::RX ? vget<T>(a, e) : T(0);
      T ye = Op::RY ? vget<T>(b, e) : T(0);
      op(xe, ye);
      if (Op::WX) vset<T>(a, e, xe);
      if (Op::WY) vset<T>(b, e, ye);
    }
    if (Op::WX) __stcs(xv + v, a);
    if (Op::WY) __stcs(yv + v, b);
  }
  if (blockIdx.x == 0) {
    const int t = threadIdx.x;
    long i = -1;
    if (t < head) i = t;
    else if (t - head < n - tail) i = tail + (t - head);
    if (i >= 0 && i < n) {
      T xe = Op::RX ? x[i] : T(0);
      T ye = Op::RY ? y[i] : T(0);
      op(xe, ye);
      if (Op::WX) x[i] = xe;
      if (Op::WY) y[i] = ye;
    }
  }
}

template <typename T, class Op>
__global__ void __launch_bounds__(kThreads) map_strided(long n, T *x, long incx, T *y, long incy, Op op) {
  const long stride = long(gridDim.x) * kThreads;
  for (long i = long(blockIdx.x) * kThreads + threadIdx.x; i < n; i += stride) {
    T xe = Op::RX ? x[i * incx] : T(0);
    T ye = Op::RY ? y[i * incy] : T(0);
    op(xe, ye);
    if (Op::WX) x[i * incx] = xe;
    if (Op::WY) y[i * incy] = ye;
  }
}

template <typename T>
int misalign(const T *p) {
  return int((reinterpret_cast<uintptr_t>(p) & 15u) / sizeof(T));
}

template <typename T, class Op>
void run_map(long n, T *x, long incx, T *y, long incy, Op op) {
  if (n <= 0) return;
  cudaStream_t s = ctx().stream;
  constexpr int VN = V16<T>::N;
  const bool unit = (!Op::RX && !Op::WX || incx == 1) && (!Op::RY && !Op::WY || incy == 1);
  // both operands must reach 16-byte alignment after the same head
  int head = -1;
  if (unit) {
    const bool hx = Op::RX || Op::WX, hy = Op::RY || Op::WY;
    const int mx = hx ? misalign(x) : -1, my = hy ? misalign(y) : -1;
    const bool xok = !hx || (reinterpret_cast<uintptr_t>(x) % sizeof(T)) == 0;
    const bool yok = !hy || (reinterpret_cast<uintptr_t>(y) % sizeof(T)) == 0;
    if (xok && yok && (!hx || !hy || mx == my)) {
      const int m = hx ? mx : my;
      head = m == 0 ? 0 : VN - m;
      if (head > n) head = int(n);
    }
  }
  if (head >= 0) {
    const long nvec = (n - head) / VN;
    long blocks = ceil_div(nvec, long(kThreads) * kUnroll);
    if (blocks < 1) blocks = 1;
    if (blocks > grid_cap(8)) blocks = grid_cap(8);
    map_unit<T, Op><<<int(blocks), kThreads, 0, s>>>(n, x, y, op, head);
  } else {
    long blocks = ceil_div(n, long(kThreads) * 4);
    if (blocks > grid_cap(8)) blocks = grid_cap(8);
    map_strided<T, Op><<<int(blocks), kThreads, 0, s>>>(n, x, incx, y, incy, op);
  }
  EXB_LAUNCH("level-1 map kernel");
  count_launch();
}

template <typename T>
void axpy(long n, T alpha, const T *x, long incx, T *y, long incy) {
  T *xm = const_cast<T *>(x);
  if (alpha == T(1) && incx == 1 && incy == 1)  // exo_axpy_wrapper.h:12-15
    run_map(n, xm, incx, y, incy, Axpy1Op<T>{});
  else
    run_map(n, xm, incx, y, incy, AxpyOp<T>{alpha});
}
template <typename T>
void scal(long n, T alpha, T *x, long incx) {
  if (alpha == T(0))
    run_map(n, x, incx, x, incx, ScalZeroOp<T>{});
  else
    run_map(n, x, incx, x, incx, ScalOp<T>{alpha});
}
template <typename T>
void copy(long n, const T *x, long incx, T *y, long incy) {
  run_map(n, const_cast<T *>(x), incx, y, incy, CopyOp<T>{});
}
template <typename T>
void swap(long n, T *x, long incx, T *y, long incy) {
  run_map(n, x, incx, y, incy, SwapOp<T>{});
}
template <typename T>
void rot(long n, T *x, long incx, T *y, long incy, T c, T s) {
  run_map(n, x, incx, y, incy, RotOp<T>{c, s});
}
template <typename T>
void rotm(long n, T *x, long incx, T *y, long incy, const T P[5]) {
  // H = {P[1], P[3], P[2], P[4]} row-major (exo_rotm_wrapper.h:8)
  const T flag = P[0], h00 = P[1], h01 = P[3], h10 = P[2], h11 = P[4];
  if (flag == T(-1))
    run_map(n, x, incx, y, incy, RotmNegOneOp<T>{h00, h01, h10, h11});
  else if (flag == T(0))
    run_map(n, x, incx, y, incy, RotmZeroOp<T>{h01, h10});
  else if (flag == T(1))
    run_map(n, x, incx, y, incy, RotmOneOp<T>{h00, h11});
}

// -------------------------------------------------------------- reductions --

// Accumulators.  sasum / dot accumulate in the working precision (T)
// (dasum: integer significand sums in level1_ext.cu); dsdot
// accumulates exact products x*y = p + e (p = fl(x*y), e = fma(x, y, -p))
// in an unevaluated float pair (hi, lo) updated by TwoSum, so the FP32 pipe
// carries the per-element work; block and grid sums are native FP64.
template <typename T>
struct AsumAcc {
  using In = T;
  using Part = T;
  using Out = T;
  static constexpr bool TWO = false;
  T s = 0;
  __device__ void add(T x, T) { s += fabs(x); }
  __device__ Part part() const { return s; }
};
template <typename T>
struct DotAcc {
  using In = T;
  using Part = T;
  using Out = T;
  static constexpr bool TWO = true;
  T s = 0;
  __device__ void add(T x, T y) { s = fma(x, y, s); }
  __device__ Part part() const { return s; }
};
struct DsdotAcc {
  using In = float;
  using Part = double;
  using Out = double;
  static constexpr bool TWO = true;
  float hi = 0.f, lo = 0.f;
  __device__ void add(float x, float y) {
    const float p = x * y;
    const float e = fmaf(x, y, -p);
    const float s = hi + p;
    const float z = s - hi;
    const float err = (hi - (s - z)) + (p - z);
    hi = s;
    lo += err + e;
  }
  __device__ Part part() const { return double(hi) + double(lo); }
};

template <class Acc>
__global__ void __launch_bounds__(kThreads)
    reduce_kernel(long n, const typename Acc::In *__restrict__ x, long incx, const typename Acc::In *__restrict__ y,
                  long incy, int head, bool unit, typename Acc::Part *partials, unsigned int *counter,
                  typename Acc::Out *result, float sb, float *sresult) {
  using T = typename Acc::In;
  using P = typename Acc::Part;
  using V = typename V16<T>::type;
  constexpr int VN = V16<T>::N;
  __shared__ P sh[kThreads / 32];
  __shared__ bool last;
  Acc acc;
  const long stride = long(gridDim.x) * kThreads;
  const long gt = long(blockIdx.x) * kThreads + threadIdx.x;
  if (unit) {
    const long nvec = (n - head) / VN;
    const long tail = head + nvec * VN;
    const V *xv = reinterpret_cast<const V *>(x + head);
    const V *yv = reinterpret_cast<const V *>(y + head);
    long v = gt;
    // software pipeline: the next kU vectors (of x and y) are loaded
    // before the current ones are consumed; one-operand reductions keep
    // twice as many vectors per thread in flight.  Two register buffers
    // alternate (the body is written twice), so no vector is copied between
    // registers; measured faster than copying the prefetched buffer (ddot
    // 0.90 -> 0.95 of the HBM copy bandwidth on GB300).
    constexpr int kU = Acc::TWO ? kUnroll : 2 * kUnroll;
    V a0[kU], b0[kU], a1[kU], b1[kU];
    auto load = [&](V(&xa)[kU], V(&ya)[kU], long at) {
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        xa[u] = ld_stream(xv + at + u * stride);
        if (Acc::TWO) ya[u] = ld_stream(yv + at + u * stride);
      }
    };
    auto use = [&](V(&xa)[kU], V(&ya)[kU]) {
#pragma unroll
      for (int u = 0; u < kU; ++u)
#pragma unroll
        for (int e = 0; e < VN; ++e) acc.add(vget<T>(xa[u], e), Acc::TWO ? vget<T>(ya[u], e) : T(0));
    };
    bool have = v + (kU - 1) * stride < nvec;
    if (have) load(a0, b0, v);
    while (have) {
      long vn = v + kU * stride;
      bool more = vn + (kU - 1) * stride < nvec;
      if (more) load(a1, b1, vn);
      use(a0, b0);
      v = vn;
      if (!more) break;
      vn = v + kU * stride;
      more = vn + (kU - 1) * stride < nvec;
      if (more) load(a0, b0, vn);
      use(a1, b1);
      v = vn;
      have = more;
    }
    for (; v < nvec; v += stride) {
      V a = ld_stream(xv + v), b;
      if (Acc::TWO) b = ld_stream(yv + v);
#pragma unroll
      for (int e = 0; e < VN; ++e) acc.add(vget<T>(a, e), Acc::TWO ? vget<T>(b, e) : T(0));
    }
    if (blockIdx.x == 0) {
      const int t = threadIdx.x;
      long i = -1;
      if (t < head) i = t;
      else if (t - head < n - tail) i = tail + (t - head);
      if (i >= 0 && i < n) acc.add(x[i], Acc::TWO ? y[i] : T(0));
    }
  } else {
    for (long i = gt; i < n; i += stride) acc.add(x[i * incx], Acc::TWO ? y[i * incy] : T(0));
  }
  P total = block_sum<P>(acc.part(), sh);
  if (gridDim.x > 1) {
    if (threadIdx.x == 0) {
      partials[blockIdx.x] = total;
      __threadfence();
      const unsigned int ticket = atomicAdd(counter, 1u);
      last = ticket == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    P s = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) s += __ldcg(partials + b);
    total = block_sum<P>(s, sh);
    if (threadIdx.x == 0) *counter = 0;  // leave the counter zero for the next call
  }
  if (threadIdx.x == 0) {
    *result = total;
    if (sresult) {  // dsdot.py:33-36: d_result = d_dot + sb, rounded to float
      double d = double(total) + double(sb);
      *sresult = float(d);
    }
  }
}

template <class Acc>
void run_reduce(long n, const typename Acc::In *x, long incx, const typename Acc::In *y, long incy,
                typename Acc::Out *result, float sb = 0.f, float *sresult = nullptr) {
  using T = typename Acc::In;
  using P = typename Acc::Part;
  constexpr int VN = V16<T>::N;
  cudaStream_t s = ctx().stream;
  if (n < 0) n = 0;
  bool unit = incx == 1 && (!Acc::TWO || incy == 1);
  int head = 0;
  if (unit) {
    const int mx = misalign(x), my = Acc::TWO ? misalign(y) : mx;
    const bool elem_ok = reinterpret_cast<uintptr_t>(x) % sizeof(T) == 0 &&
                         (!Acc::TWO || reinterpret_cast<uintptr_t>(y) % sizeof(T) == 0);
    if (elem_ok && mx == my) {
      head = mx == 0 ? 0 : VN - mx;
      if (head > n) head = int(n);
    } else {
      unit = false;
    }
  }
  long work = unit ? (n / VN) : n;
  long blocks = ceil_div(work, long(kThreads) * kUnroll);
  if (blocks < 1) blocks = 1;
  // one wave of resident CTAs at most
  const int per_sm = resident_per_sm(reinterpret_cast<const void *>(reduce_kernel<Acc>), kThreads);
  if (blocks > grid_cap(per_sm < 4 ? per_sm : 4)) blocks = grid_cap(per_sm < 4 ? per_sm : 4);
  P *partials = static_cast<P *>(scratch(sizeof(P) * blocks));
  unsigned int *counter = zero_words(1);
  reduce_kernel<Acc><<<int(blocks), kThreads, 0, s>>>(n, x, incx, y, incy, head, unit, partials, counter, result, sb,
                                                     sresult);
  EXB_LAUNCH("level-1 reduction kernel");
  count_launch();
}

template <typename T>
void asum(long n, const T *x, long incx, T *result) {
  if constexpr (sizeof(T) == 8)
    dasum_words(n, x, incx, result);
  else
    run_reduce<AsumAcc<T>>(n, x, incx, x, incx, result);
}
template <typename T>
void dot(long n, const T *x, long incx, const T *y, long incy, T *result) {
  run_reduce<DotAcc<T>>(n, x, incx, y, incy, result);
}
void dsdot(long n, const float *x, long incx, const float *y, long incy, double *result, float sb, float *sresult) {
  run_reduce<DsdotAcc>(n, x, incx, y, incy, result, sb, sresult);
}

#define EXB_L1_INST(T)                                                           \
  template void axpy<T>(long, T, const T *, long, T *, long);                    \
  template void scal<T>(long, T, T *, long);                                     \
  template void copy<T>(long, const T *, long, T *, long);                       \
  template void swap<T>(long, T *, long, T *, long);                             \
  template void rot<T>(long, T *, long, T *, long, T, T);                        \
  template void rotm<T>(long, T *, long, T *, long, const T *);                  \
  template void asum<T>(long, const T *, long, T *);                             \
  template void dot<T>(long, const T *, long, const T *, long, T *);
EXB_L1_INST(float)
EXB_L1_INST(double)

}  // namespace l1
}  // namespace exb
