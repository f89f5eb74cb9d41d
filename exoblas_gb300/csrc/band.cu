// Banded level 2: gbmv, sbmv, tbmv (one row-parallel kernel) and tbsv.
//
// Band storage is the row-major CBLAS layout the reference's procs index:
//   general (kl, ku)  A(r, c) at a[r * lda + (c - r + kl)],  -kl <= c - r <= ku
//   upper (k)         A(r, c) at a[r * lda + (c - r)],        0 <= c - r <= k
//   lower (k)         A(r, c) at a[r * lda + k - (r - c)],    0 <= r - c <= k
// Reference algorithms: src/level2/{gbmv,sbmv,tbmv,tbsv}.py.
//
// band_mv_kernel: a group of G lanes per output row walks the row's band
// offsets d = c - i, accumulates in lane order and reduces with a fixed
// shuffle tree (deterministic).  The general and the triangular NoTrans
// bands are contiguous in a row of `a`; the symmetric and transposed ones
// read the mirrored entries down a diagonal of the storage.  HBM-bound: the
// band is read once (twice for sbmv's mirrored half, mostly from L2).
// tbsv_kernel: one warp per system, rows in dependency order, the band dot
// of each row split over the lanes, the division by the pivot as in the
// reference.
#include <cuda_runtime.h>

#include "common.cuh"
#include "gemv_kernels.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace l2 {

namespace bd {

enum Mode { kGeneral = 0, kSymmetric = 1, kTriangular = 2 };
constexpr int kUpperBit = 1, kTransBit = 2, kUnitBit = 4;

// element (i, i + d) of the operator the row kernel applies
template <typename T, int MODE>
__device__ __forceinline__ T elem(const T *a, long lda, long i, long d, long kl, long k, int flags) {
  const bool upper = flags & kUpperBit;
  if (MODE == kGeneral) return a[i * lda + d + kl];
  if (MODE == kSymmetric) {
    if (upper) return d >= 0 ? a[i * lda + d] : a[(i + d) * lda - d];
    return d <= 0 ? a[i * lda + k + d] : a[(i + d) * lda + k - d];
  }
  // triangular op(A)(i, i + d)
  if (d == 0 && (flags & kUnitBit)) return T(1);
  if (!(flags & kTransBit)) return upper ? a[i * lda + d] : a[i * lda + k + d];
  return upper ? a[(i + d) * lda - d] : a[(i + d) * lda + k - d];
}

// band offsets [dlo, dhi] of row i's operator row
template <int MODE>
__device__ __forceinline__ void row_band(long kl, long ku, int flags, long &dlo, long &dhi) {
  if (MODE == kGeneral) {
    dlo = -kl;
    dhi = ku;
  } else if (MODE == kSymmetric) {
    dlo = -kl;
    dhi = kl;
  } else {
    const bool up_side = bool(flags & kUpperBit) != bool(flags & kTransBit);
    dlo = up_side ? 0 : -kl;
    dhi = up_side ? kl : 0;
  }
}

// kGeneral / kSymmetric: y[i] = beta y[i] + alpha (row i . x)
// kTriangular:          y[i] = row i . x (x is a copy; y the caller's x)
template <typename T, int G, int MODE>
__global__ void __launch_bounds__(kThreads)
    band_mv_kernel(long rows, long cols, long kl, long ku, T alpha, const T *__restrict__ a, long lda,
                   const T *__restrict__ x, T beta, T *y, long incy, int flags) {
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31, sub = lane % G;
  const long warp = (long(blockIdx.x) * kThreads + threadIdx.x) / 32;
  const long nwarps = long(gridDim.x) * (kThreads / 32);
  long dlo0, dhi0;
  row_band<MODE>(kl, ku, flags, dlo0, dhi0);
  for (long base = warp * RPW; base < rows; base += nwarps * RPW) {
    const long i = base + lane / G;
    T acc = T(0);
    if (i < rows) {
      const long dlo = dlo0 > -i ? dlo0 : -i;
      const long dhi = dhi0 < cols - 1 - i ? dhi0 : cols - 1 - i;
      for (long d = dlo + sub; d <= dhi; d += G) acc = fma(elem<T, MODE>(a, lda, i, d, kl, kl, flags), x[i + d], acc);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (i < rows && sub == 0) {
      T *yi = y + i * incy;
      *yi = MODE == kTriangular ? acc : beta * *yi + alpha * acc;
    }
  }
}

// op(A) x = b in place, one warp: forward when the operator is lower
// triangular (Lower/NoTrans, Upper/Trans), backward otherwise.  xs holds
// the solution as it forms (unit stride); x (stride incx) receives it too.
template <typename T>
__global__ void __launch_bounds__(32) tbsv_kernel(long n, long k, const T *__restrict__ a, long lda, T *xs, T *x,
                                                  long incx, int flags) {
  const int lane = threadIdx.x;
  const bool forward = bool(flags & kUpperBit) == bool(flags & kTransBit);
  for (long s = 0; s < n; ++s) {
    const long i = forward ? s : n - 1 - s;
    // solved neighbours: forward c in [i-k, i-1], backward c in [i+1, i+k]
    long dlo = forward ? -k : 1, dhi = forward ? -1 : k;
    if (dlo < -i) dlo = -i;
    if (dhi > n - 1 - i) dhi = n - 1 - i;
    T dot = T(0);
    for (long d = dlo + lane; d <= dhi; d += 32)
      dot = fma(elem<T, kTriangular>(a, lda, i, d, k, k, flags & ~kUnitBit), xs[i + d], dot);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
    if (lane == 0) {
      const T pivot = (flags & kUnitBit) ? T(1) : elem<T, kTriangular>(a, lda, i, 0, k, k, flags & ~kUnitBit);
      const T xi = (xs[i] - dot) / pivot;
      xs[i] = xi;
      if (x != xs) x[i * incx] = xi;
    }
    __syncwarp();
  }
}

template <typename T>
static void pack(long n, const T *src, long inc, T *dst) {
  if (n <= 0) return;
  long blocks = ceil_div(n, kThreads);
  if (blocks > grid_cap(4)) blocks = grid_cap(4);
  pack_kernel<T><<<int(blocks), kThreads, 0, ctx().stream>>>(n, src, inc, dst);
  EXB_LAUNCH("pack kernel");
  count_launch();
}

template <typename T, int MODE>
static void launch(long rows, long cols, long kl, long ku, T alpha, const T *a, long lda, const T *x, T beta, T *y,
                   long incy, int flags) {
  if (rows <= 0) return;
  const long width = MODE == kGeneral ? kl + ku + 1 : (MODE == kSymmetric ? 2 * kl + 1 : kl + 1);
  const int G = width >= 48 ? 32 : 4;
  const long rpb = (kThreads / 32) * (32 / G);
  long blocks = ceil_div(rows, rpb);
  if (blocks > grid_cap(16)) blocks = grid_cap(16);
  if (G == 32)
    band_mv_kernel<T, 32, MODE><<<int(blocks), kThreads, 0, ctx().stream>>>(rows, cols, kl, ku, alpha, a, lda, x, beta,
                                                                          y, incy, flags);
  else
    band_mv_kernel<T, 4, MODE><<<int(blocks), kThreads, 0, ctx().stream>>>(rows, cols, kl, ku, alpha, a, lda, x, beta,
                                                                         y, incy, flags);
  EXB_LAUNCH("band matrix-vector kernel");
  count_launch();
}

}  // namespace bd

// src/level2/gbmv.py:12-50: y = beta y + alpha A x, A general banded m x n
template <typename T>
void gbmv(long m, long n, long kl, long ku, T alpha, const T *A, long lda, const T *x, long incx, T beta, T *y,
          long incy) {
  if (m <= 0) return;
  const T *xu = x;
  if (n > 0 && (incx != 1 || !aligned16(x))) {
    T *tmp = static_cast<T *>(scratch(sizeof(T) * size_t(n)));
    bd::pack(n, x, incx, tmp);
    xu = tmp;
  }
  bd::launch<T, bd::kGeneral>(m, n, kl, ku, alpha, A, lda, xu, beta, y, incy, 0);
}

// src/level2/sbmv.py:8-44: y = beta y + alpha A x, A symmetric banded
template <typename T>
void sbmv(bool upper, long n, long k, T alpha, const T *A, long lda, const T *x, long incx, T beta, T *y, long incy) {
  if (n <= 0) return;
  const T *xu = x;
  if (incx != 1 || !aligned16(x)) {
    T *tmp = static_cast<T *>(scratch(sizeof(T) * size_t(n)));
    bd::pack(n, x, incx, tmp);
    xu = tmp;
  }
  bd::launch<T, bd::kSymmetric>(n, n, k, k, alpha, A, lda, xu, beta, y, incy, upper ? bd::kUpperBit : 0);
}

// src/level2/tbmv.py:9-120: x = op(A) x, A triangular banded
template <typename T>
void tbmv(bool upper, bool trans, bool unit, long n, long k, const T *A, long lda, T *x, long incx) {
  if (n <= 0) return;
  T *xc = static_cast<T *>(scratch(sizeof(T) * size_t(n)));
  bd::pack(n, x, incx, xc);
  const int flags = (upper ? bd::kUpperBit : 0) | (trans ? bd::kTransBit : 0) | (unit ? bd::kUnitBit : 0);
  bd::launch<T, bd::kTriangular>(n, n, k, k, T(1), A, lda, xc, T(0), x, incx, flags);
}

// src/level2/tbsv.py:9-120: op(A) x = b in place, A triangular banded
template <typename T>
void tbsv(bool upper, bool trans, bool unit, long n, long k, const T *A, long lda, T *x, long incx) {
  if (n <= 0) return;
  T *xs = x;
  if (incx != 1) {
    xs = static_cast<T *>(scratch(sizeof(T) * size_t(n)));
    bd::pack(n, x, incx, xs);
  }
  const int flags = (upper ? bd::kUpperBit : 0) | (trans ? bd::kTransBit : 0) | (unit ? bd::kUnitBit : 0);
  bd::tbsv_kernel<T><<<1, 32, 0, ctx().stream>>>(n, k, A, lda, xs, x, incx, flags);
  EXB_LAUNCH("banded triangular solve kernel");
  count_launch();
}

#define EXB_BAND_INSTANTIATE(T)                                                                              \
  template void gbmv<T>(long, long, long, long, T, const T *, long, const T *, long, T, T *, long);          \
  template void sbmv<T>(bool, long, long, T, const T *, long, const T *, long, T, T *, long);                \
  template void tbmv<T>(bool, bool, bool, long, long, const T *, long, T *, long);                           \
  template void tbsv<T>(bool, bool, bool, long, long, const T *, long, T *, long);
EXB_BAND_INSTANTIATE(float)
EXB_BAND_INSTANTIATE(double)
#undef EXB_BAND_INSTANTIATE

}  // namespace l2
}  // namespace exb
