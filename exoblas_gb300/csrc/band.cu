// Banded level 2: gbmv, sbmv, tbmv (one row-parallel kernel) and tbsv.
//
// Band storage is the row-major CBLAS layout the reference's procs index:
//   general (kl, ku)  A(r, c) at a[r * lda + (c - r + kl)],  -kl <= c - r <= ku
//   upper (k)         A(r, c) at a[r * lda + (c - r)],        0 <= c - r <= k
//   lower (k)         A(r, c) at a[r * lda + k - (r - c)],    0 <= r - c <= k
// Reference algorithms: src/level2/{gbmv,sbmv,tbmv,tbsv}.py.
//
// band_tile_kernel (narrow bands): a CTA stages the storage rows of 64 or
// 128 output rows (plus the k mirrored rows before or after for sbmv and
// transposed tbmv) in shared memory with coalesced reads and one thread per
// output row walks its band offsets d = c - i in order.  band_mv_kernel
// (wide bands): a group of G lanes per output row walks the offsets,
// accumulates in lane order and reduces with a fixed shuffle tree.  Both
// are deterministic and read the band from HBM about once.
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

__device__ __forceinline__ void cp_async_16(void *smem, const void *gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
template <typename T>
__device__ __forceinline__ void cp_async_elem(T *smem, const T *gmem) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}

// Narrow bands: a CTA stages the storage rows its kTR output rows touch
// (the rows themselves plus, for mirrored or transposed operators, the k
// rows before or after) into shared memory with coalesced row reads, then
// one thread per output row walks its band offsets from shared memory.
template <typename T>
struct Tile {
  static constexpr int kTR = sizeof(T) == 4 ? 128 : 64;  // output rows (and threads) per CTA
};

template <typename T, int MODE>
__global__ void __launch_bounds__(Tile<T>::kTR)
    band_tile_kernel(long rows, long cols, long kl, long ku, T alpha, const T *__restrict__ a, long lda,
                     const T *__restrict__ x, T beta, T *y, long incy, int flags, int W, int lo, int hi) {
  constexpr int kTR = Tile<T>::kTR;
  extern __shared__ __align__(16) unsigned char band_smem[];
  T *tile = reinterpret_cast<T *>(band_smem);  // (kTR + lo + hi) storage rows x W
  const int k = int(kl), xw_len = kTR + int(kl) + int(ku);
  T *xw = tile + size_t(kTR + lo + hi) * W + 16 / sizeof(T);  // x[r0 - kl .. r0 + kTR + ku)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long dlo0, dhi0;
  row_band<MODE>(kl, ku, flags, dlo0, dhi0);
  const int nr = kTR + lo + hi;
  const long ntiles = ceil_div(rows, long(kTR));
  for (long t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const long r0 = t * kTR, q0 = r0 - lo;
    // storage element e of the tile lands at tb[e - q0 * lda]; tb is shifted
    // so that 16-byte aligned storage chunks land 16-byte aligned
    constexpr int kPer = 16 / int(sizeof(T));
    const int sh = lda == W ? int(((q0 * lda) % kPer + kPer) % kPer) : 0;
    T *tb = tile + sh;
    __syncthreads();  // the previous tile's reads are done
    // asynchronous copies, all in flight at once
    if (lda == W) {
      // the tile is one contiguous span of the storage: 16-byte copies for
      // its aligned body, element copies for the ends and zeros outside
      const long s0 = q0 * lda, s1 = s0 + long(nr) * W;  // storage elements [s0, s1)
      const long lo_in = s0 > 0 ? s0 : 0, hi_in = s1 < rows * lda ? s1 : rows * lda;
      long b0 = (lo_in + kPer - 1) / kPer * kPer, b1 = hi_in / kPer * kPer;
      const bool a16 = (reinterpret_cast<uintptr_t>(a) & 15u) == 0;
      if (!a16 || b1 < b0) b0 = b1 = lo_in;  // no aligned body: element copies only
      // zeros outside the storage, element copies for the unaligned ends
      for (long e = s0 + threadIdx.x; e < lo_in; e += kTR) tb[e - s0] = T(0);
      for (long e = (hi_in > s0 ? hi_in : s0) + threadIdx.x; e < s1; e += kTR) tb[e - s0] = T(0);
      for (long e = lo_in + threadIdx.x; e < b0; e += kTR) cp_async_elem(&tb[e - s0], a + e);
      for (long e = b1 + threadIdx.x; e < hi_in; e += kTR) cp_async_elem(&tb[e - s0], a + e);
      for (long c = b0 + long(threadIdx.x) * kPer; c < b1; c += long(kTR) * kPer)
        cp_async_16(&tb[c - s0], a + c);
    } else {
      for (int rr = warp; rr < nr; rr += kTR / 32) {
        const long q = q0 + rr;
        const bool in = q >= 0 && q < rows;
        for (int j = lane; j < W; j += 32) {
          if (in)
            cp_async_elem(&tb[rr * W + j], a + q * lda + j);
          else
            tb[rr * W + j] = T(0);
        }
      }
    }
    for (int e = threadIdx.x; e < xw_len; e += kTR) {
      const long c = r0 - kl + e;
      if (c >= 0 && c < cols)
        cp_async_elem(&xw[e], x + c);
      else
        xw[e] = T(0);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    const long i = r0 + threadIdx.x;
    if (i < rows) {
      const int dlo = int(dlo0 > -i ? dlo0 : -i);
      const int dhi = int(dhi0 < cols - 1 - i ? dhi0 : cols - 1 - i);
      // Along d the shared-memory address is affine on each side of the
      // diagonal: step 1 where the entry sits in row i's own storage row,
      // step W - 1 where it is mirrored from row i + d.  Two segments at most.
      const int ti = int(i - r0) + lo;  // row i's storage row within the tile
      const T *xi = xw + (int(i - r0) + k);  // xi[d] = x[i + d]
      const bool unit = MODE == kTriangular && (flags & kUnitBit);
      T acc = T(0);
      auto run = [&](int da, int db, int addr, int step) {
#pragma unroll 4
        for (int d = da; d <= db; ++d) {
          const T v = (unit && d == 0) ? T(1) : tb[addr + (d - da) * step];
          acc = fma(v, xi[d], acc);
        }
      };
      const bool upper = flags & kUpperBit;
      if (MODE == kGeneral) {
        run(dlo, dhi, ti * W + dlo + k, 1);
      } else if (MODE == kSymmetric) {
        if (upper) {  // d < 0 mirrored (j = -d), d >= 0 direct (j = d)
          run(dlo, dhi < -1 ? dhi : -1, ti * W + dlo * (W - 1), W - 1);
          run(dlo > 0 ? dlo : 0, dhi, ti * W + (dlo > 0 ? dlo : 0), 1);
        } else {  // d <= 0 direct (j = k + d), d > 0 mirrored (j = k - d)
          run(dlo, dhi < 0 ? dhi : 0, ti * W + k + dlo, 1);
          run(dlo > 1 ? dlo : 1, dhi, ti * W + k + (dlo > 1 ? dlo : 1) * (W - 1), W - 1);
        }
      } else if (!(flags & kTransBit)) {  // direct: j = d (upper), k + d (lower)
        run(dlo, dhi, ti * W + (upper ? 0 : k) + dlo, 1);
      } else {  // mirrored from row i + d: j = -d (upper), k - d (lower)
        run(dlo, dhi, ti * W + (upper ? 0 : k) + dlo * (W - 1), W - 1);
      }
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
  // narrow bands: shared-memory tiles (at most 48 KB per CTA)
  const long W = MODE == kGeneral ? kl + ku + 1 : kl + 1;  // storage row width
  const bool mirrored = MODE == kSymmetric || (MODE == kTriangular && (flags & kTransBit));
  const bool before = mirrored && (MODE == kSymmetric ? bool(flags & kUpperBit) : bool(flags & kUpperBit));
  const long lo = mirrored && before ? kl : 0, hi = mirrored && !before ? kl : 0;
  constexpr int kTR = Tile<T>::kTR;
  const size_t smem = (size_t(kTR + lo + hi) * size_t(W) + size_t(kTR + kl + ku)) * sizeof(T) + 16;
  if (smem <= 48 * 1024) {
    const long ntiles = ceil_div(rows, long(kTR));
    const int per_sm = resident_per_sm(reinterpret_cast<const void *>(band_tile_kernel<T, MODE>), kTR, smem);
    long blocks = ntiles < long(ctx().sm_count) * per_sm ? ntiles : long(ctx().sm_count) * per_sm;
    band_tile_kernel<T, MODE><<<int(blocks), kTR, smem, ctx().stream>>>(rows, cols, kl, ku, alpha, a, lda, x, beta, y,
                                                                       incy, flags, int(W), int(lo), int(hi));
    EXB_LAUNCH("band tile kernel");
    count_launch();
    return;
  }
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
