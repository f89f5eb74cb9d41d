// Level-2 kernels (gemv, ger, symv, syr, syr2, trmv): each streams the
// matrix from HBM once with 16-byte loads.  Reductions across CTAs go
// through per-chunk partial rows in scratch that a second kernel sums in a
// fixed order, so results are deterministic.
// Reference algorithms: src/level2/{gemv,ger,symv,syr,syr2,trmv}.py.
#include <cuda_runtime.h>

#include "common.cuh"
#include "gemv_kernels.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace l2 {

// Carves one scratch allocation into 256-byte aligned regions.
struct Carve {
  size_t off = 0;
  char *base = nullptr;
  template <typename T>
  size_t add(long n) {
    size_t o = off;
    off += (size_t(n > 0 ? n : 1) * sizeof(T) + 255) & ~size_t(255);
    return o;
  }
  void alloc() { base = static_cast<char *>(scratch(off)); }
  template <typename T>
  T *at(size_t o) const {
    return reinterpret_cast<T *>(base + o);
  }
};

template <typename T>
static bool vec_ok(const T *A, long lda) {
  return aligned16(A) && (lda * long(sizeof(T))) % 16 == 0;
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

// Returns a unit-stride, 16-byte aligned view of x (packing into `tmp` when needed).
template <typename T>
static const T *unit_view(long n, const T *x, long inc, T *tmp) {
  if (inc == 1 && aligned16(x)) return x;
  pack(n, x, inc, tmp);
  return tmp;
}

template <typename T, int MODE>
static void launch_rowdot(long rows, long cols, T alpha, const T *A, long lda, const T *xu, T beta, T *y, long incy,
                          int tri, bool unit) {
  cudaStream_t s = ctx().stream;
  const bool vec = vec_ok(A, lda) && aligned16(xu);
  const int G = cols >= 256 ? 32 : 4;
  const long rpb = (kThreads / 32) * (32 / G);
  // whole waves of equal row counts per warp (no partial last wave)
  const void *kern = G == 32 ? (vec ? reinterpret_cast<const void *>(rowdot_kernel<T, 32, true, MODE>)
                                    : reinterpret_cast<const void *>(rowdot_kernel<T, 32, false, MODE>))
                             : (vec ? reinterpret_cast<const void *>(rowdot_kernel<T, 4, true, MODE>)
                                    : reinterpret_cast<const void *>(rowdot_kernel<T, 4, false, MODE>));
  const long blocks = balanced_grid(ceil_div(rows, rpb), kern, kThreads);
#define EXB_ROWDOT(GG, VV) \
  rowdot_kernel<T, GG, VV, MODE><<<int(blocks), kThreads, 0, s>>>(rows, cols, alpha, A, lda, xu, beta, y, incy, tri, unit)
  if (G == 32) {
    if (vec) EXB_ROWDOT(32, true);
    else EXB_ROWDOT(32, false);
  } else {
    if (vec) EXB_ROWDOT(4, true);
    else EXB_ROWDOT(4, false);
  }
#undef EXB_ROWDOT
  EXB_LAUNCH("row-dot kernel");
  count_launch();
}

template <typename T>
static int colsum_chunks(long rows, long cols) {
  constexpr int VN = V16<T>::N;
  const long tiles = ceil_div(cols, 32 * VN);
  long chunks = ceil_div(grid_cap(4), tiles);
  const long max_chunks = ceil_div(rows, 64);
  if (chunks > max_chunks) chunks = max_chunks;
  if (chunks < 1) chunks = 1;
  return int(chunks);
}

template <typename T>
static void launch_colsum(long rows, long cols, const T *A, long lda, const T *xu, int chunks, T *partial, int tri,
                          bool unit) {
  constexpr int VN = V16<T>::N;
  const long rpc = ceil_div(rows, chunks);
  dim3 grid(unsigned(ceil_div(cols, 32 * VN)), unsigned(chunks));
  if (vec_ok(A, lda))
    colsum_kernel<T, true><<<grid, kThreads, 0, ctx().stream>>>(rows, cols, A, lda, xu, rpc, partial, tri, unit);
  else
    colsum_kernel<T, false><<<grid, kThreads, 0, ctx().stream>>>(rows, cols, A, lda, xu, rpc, partial, tri, unit);
  EXB_LAUNCH("column-sum kernel");
  count_launch();
}

template <typename T, int MODE>
static void launch_finish(long cols, int chunks, const T *partial, T alpha, T beta, T *y, long incy, const T *xs,
                          bool unit) {
  const long blocks = finish_blocks(cols, grid_cap(8));
  finish_kernel<T, MODE><<<int(blocks), kThreads, 0, ctx().stream>>>(cols, chunks, partial, alpha, beta, y, incy, xs,
                                                                     unit);
  EXB_LAUNCH("partial-sum kernel");
  count_launch();
}

// src/level2/gemv.py:10-22.  rows x cols is the caller's M x N matrix.
template <typename T>
void gemv(bool trans, long rows, long cols, T alpha, const T *A, long lda, const T *x, long incx, T beta, T *y,
          long incy) {
  if (rows <= 0 && cols <= 0) return;
  const long xlen = trans ? rows : cols, ylen = trans ? cols : rows;
  if (ylen <= 0) return;
  if (xlen <= 0) {
    // y = beta * y (gemv.py:13-14) with nothing to add
    l1::scal<T>(ylen, beta, y, incy);
    return;
  }
  Carve cv;
  const size_t ox = cv.add<T>(xlen);
  const int chunks = trans ? colsum_chunks<T>(rows, cols) : 0;
  const size_t op = trans ? cv.add<T>(long(chunks) * cols) : 0;
  cv.alloc();
  const T *xu = unit_view(xlen, x, incx, cv.at<T>(ox));
  if (!trans) {
    launch_rowdot<T, 0>(rows, cols, alpha, A, lda, xu, beta, y, incy, 0, false);
  } else {
    T *partial = cv.at<T>(op);
    launch_colsum<T>(rows, cols, A, lda, xu, chunks, partial, 0, false);
    launch_finish<T, 0>(cols, chunks, partial, alpha, beta, y, incy, nullptr, false);
  }
}

// src/level2/trmv.py:9-43: x = op(A) x with A triangular.
template <typename T>
void trmv(bool upper, bool trans, bool unit, long n, const T *A, long lda, T *x, long incx) {
  if (n <= 0) return;
  Carve cv;
  const size_t ox = cv.add<T>(n);
  const int chunks = trans ? colsum_chunks<T>(n, n) : 0;
  const size_t op = trans ? cv.add<T>(long(chunks) * n) : 0;
  cv.alloc();
  T *xs = cv.at<T>(ox);
  pack(n, x, incx, xs);  // the kernels read this copy; x is the output
  const int tri = upper ? 2 : 1;
  if (!trans) {
    launch_rowdot<T, 1>(n, n, T(1), A, lda, xs, T(0), x, incx, tri, unit);
  } else {
    T *partial = cv.at<T>(op);
    launch_colsum<T>(n, n, A, lda, xs, chunks, partial, tri, unit);
    launch_finish<T, 1>(n, chunks, partial, T(1), T(0), x, incx, xs, unit);
  }
}

// ---------------------------------------------------------- rank updates --
// One CTA per row (grid-stride): the row's columns [lo, hi) are updated in
// 16-byte vectors with scalar head/tail.  MODE 0 ger, 1 syr, 2 syr2.
template <typename T, bool VEC, int MODE>
__global__ void __launch_bounds__(kThreads)
    rank_kernel(long rows, long cols, T alpha, const T *__restrict__ x, const T *__restrict__ y, T *A, long lda,
                int tri) {
  using V = typename V16<T>::type;
  constexpr int VN = V16<T>::N;
  long pass = 0;
  for (long q = blockIdx.x; q < rows; q += gridDim.x, ++pass) {
    long i = q;
    if (tri != 0 && (pass & 1)) {
      // triangle rows snake (odd passes mirrored) for equal work per CTA
      const long cs = pass * gridDim.x;
      const long ce = cs + gridDim.x < rows ? cs + gridDim.x : rows;
      i = ce - 1 - (q - cs);
    }
    long lo = 0, hi = cols;
    if (tri == 1) hi = i + 1;  // lower
    if (tri == 2) lo = i;      // upper
    T *a = A + i * lda;
    const T ax = alpha * x[i];                  // ger.py:15, syr.py:17-19
    const T ay = MODE == 2 ? alpha * y[i] : T(0);  // syr2.py:25-27
    const T *u = MODE == 1 ? x : y;
    auto upd = [&](T av, long j) -> T {
      // two FMAs per element: the FP64 pipe, not HBM, bounds dsyr2 on GB300
      if (MODE == 2) return fma(ay, x[j], fma(ax, y[j], av));
      return av + ax * u[j];
    };
    if (VEC) {
      // the row's own alignment (any lda): scalar head up to the first
      // 16-byte boundary at or after lo, vectors, scalar tail
      const int mis = int((reinterpret_cast<uintptr_t>(a + lo) & 15u) / sizeof(T));
      long vlo = lo + (mis ? VN - mis : 0);
      if (vlo > hi) vlo = hi;
      const long nv = (hi - vlo) / VN, vhi = vlo + nv * VN;
      for (long j = lo + threadIdx.x; j < vlo; j += kThreads) a[j] = upd(a[j], j);
      V *av = reinterpret_cast<V *>(a + vlo);
      // FP32: x and y as 16-byte vectors too when the row's vectors line up
      // with theirs, and two A vectors in flight per thread
      const bool xyv = ((reinterpret_cast<uintptr_t>(x + vlo) | reinterpret_cast<uintptr_t>(y + vlo)) & 15u) == 0;
      auto upd4 = [&](V t, long v) -> V {
        if (xyv) {
          const V xv = reinterpret_cast<const V *>(x + vlo)[v];
          const V yv = reinterpret_cast<const V *>(y + vlo)[v];
#pragma unroll
          for (int e = 0; e < VN; ++e) {
            const T ae = vget<T>(t, e);
            T r;
            if (MODE == 2)
              r = fma(ay, vget<T>(xv, e), fma(ax, vget<T>(yv, e), ae));
            else
              r = ae + ax * vget<T>(MODE == 1 ? xv : yv, e);
            vset<T>(t, e, r);
          }
        } else {
#pragma unroll
          for (int e = 0; e < VN; ++e) vset<T>(t, e, upd(vget<T>(t, e), vlo + v * VN + e));
        }
        return t;
      };
      long v = threadIdx.x;
      if constexpr (sizeof(T) == 4) {
        // FP32 only: measured slower for FP64 rows (dger 0.89 -> 0.82 of HBM)
        for (; v + kThreads < nv; v += 2 * kThreads) {
          const V t0 = av[v], t1 = av[v + kThreads];
          av[v] = upd4(t0, v);
          av[v + kThreads] = upd4(t1, v + kThreads);
        }
        for (; v < nv; v += kThreads) av[v] = upd4(av[v], v);
      } else {
        for (; v < nv; v += kThreads) {
          V t = av[v];
#pragma unroll
          for (int e = 0; e < VN; ++e) vset<T>(t, e, upd(vget<T>(t, e), vlo + v * VN + e));
          av[v] = t;
        }
      }
      for (long j = vhi + threadIdx.x; j < hi; j += kThreads) a[j] = upd(a[j], j);
    } else {
      for (long j = lo + threadIdx.x; j < hi; j += kThreads) a[j] = upd(a[j], j);
    }
  }
}

template <typename T, int MODE>
static void launch_rank(long rows, long cols, T alpha, const T *xu, const T *yu, T *A, long lda, int tri) {
  long blocks = rows;
  if (blocks > grid_cap(8)) blocks = grid_cap(8);
  // vector path whenever A is element-aligned (each row finds its own
  // head), except FP64 syr2 on rows of mixed alignment: that update is bound
  // by FP64 issue and its element path measured 6% faster (n = 11585)
  const bool elem_aligned = reinterpret_cast<uintptr_t>(A) % sizeof(T) == 0;
  if (vec_ok(A, lda) || (elem_aligned && !(MODE == 2 && sizeof(T) == 8)))
    rank_kernel<T, true, MODE><<<int(blocks), kThreads, 0, ctx().stream>>>(rows, cols, alpha, xu, yu, A, lda, tri);
  else
    rank_kernel<T, false, MODE><<<int(blocks), kThreads, 0, ctx().stream>>>(rows, cols, alpha, xu, yu, A, lda, tri);
  EXB_LAUNCH("rank-update kernel");
  count_launch();
}

// src/level2/ger.py:9-15
template <typename T>
void ger(long m, long n, T alpha, const T *x, long incx, const T *y, long incy, T *A, long lda) {
  if (m <= 0 || n <= 0) return;
  Carve cv;
  const size_t ox = cv.add<T>(m), oy = cv.add<T>(n);
  cv.alloc();
  const T *xu = unit_view(m, x, incx, cv.at<T>(ox));
  const T *yu = unit_view(n, y, incy, cv.at<T>(oy));
  launch_rank<T, 0>(m, n, alpha, xu, yu, A, lda, 0);
}

// src/level2/syr.py:10-19
template <typename T>
void syr(bool upper, long n, T alpha, const T *x, long incx, T *A, long lda) {
  if (n <= 0) return;
  Carve cv;
  const size_t ox = cv.add<T>(n);
  cv.alloc();
  const T *xu = unit_view(n, x, incx, cv.at<T>(ox));
  launch_rank<T, 1>(n, n, alpha, xu, xu, A, lda, upper ? 2 : 1);
}

// src/level2/syr2.py:9-27
template <typename T>
void syr2(bool upper, long n, T alpha, const T *x, long incx, const T *y, long incy, T *A, long lda) {
  if (n <= 0) return;
  Carve cv;
  const size_t ox = cv.add<T>(n), oy = cv.add<T>(n);
  cv.alloc();
  const T *xu = unit_view(n, x, incx, cv.at<T>(ox));
  const T *yu = unit_view(n, y, incy, cv.at<T>(oy));
  launch_rank<T, 2>(n, n, alpha, xu, yu, A, lda, upper ? 2 : 1);
}

// ------------------------------------------------------------------- symv --
// src/level2/symv.py:10-35.  The stored triangle is cut into 64 x 64 tiles;
// a CTA walks a strip of kSymStrip consecutive tiles of one storage tile
// row, reading each tile once: the tile's row contribution (A_t x_cols)
// accumulates across the strip in registers, its column contribution
// (A_t^T x_rows, off-diagonal tiles) is written at once.  Output row tile r
// receives one contribution per tile index c (slot c): P[c][rows of r]; a
// strip's row sum goes to the slot of its first tile and its other slots
// of that row tile are zero.  A second kernel sums the slots in order.
constexpr int kSymTile = 64;
constexpr int kSymStrip = 4;

template <typename T, bool VEC, int PASSES, int VN, int RPP>
__device__ __forceinline__ void symv_load(T (&av)[PASSES][VN], long n, long r0, long c0e, const T *__restrict__ A,
                                          long lda) {
  using V = typename V16<T>::type;
#pragma unroll
  for (int p = 0; p < PASSES; ++p) {
    const long r = r0 + p * RPP;
    if (r < n && VEC && c0e + VN <= n) {
      const V v = ld_stream(reinterpret_cast<const V *>(A + r * lda + c0e));
#pragma unroll
      for (int e = 0; e < VN; ++e) av[p][e] = vget<T>(v, e);
    } else {
#pragma unroll
      for (int e = 0; e < VN; ++e) av[p][e] = (r < n && c0e + e < n) ? A[r * lda + c0e + e] : T(0);
    }
  }
}

// One tile's products: row partials accumulate in rowacc (per pass, over
// this thread's columns), column partials in colacc.  DIAG masks the half of
// a diagonal tile outside the stored triangle (and its diagonal for the
// column product, which the row product already holds).
template <bool DIAG, typename T, int PASSES, int VN, int RPP>
__device__ __forceinline__ void symv_tile(T (&av)[PASSES][VN], T (&xc)[VN], T (&xr)[PASSES],
                                          T (&rowacc)[PASSES], T (&colacc)[VN], int cl, int rl, bool upper) {
#pragma unroll
  for (int p = 0; p < PASSES; ++p) {
    const int r = rl + p * RPP;  // row within the tile
#pragma unroll
    for (int e = 0; e < VN; ++e) {
      const int c = cl + e;  // column within the tile
      const T a = av[p][e];
      if (DIAG) {
        const bool in_row = upper ? c >= r : c <= r;
        const bool in_col = upper ? c > r : c < r;
        rowacc[p] = fma(in_row ? a : T(0), xc[e], rowacc[p]);
        colacc[e] = fma(in_col ? a : T(0), xr[p], colacc[e]);
      } else {
        rowacc[p] = fma(a, xc[e], rowacc[p]);
        colacc[e] = fma(a, xr[p], colacc[e]);
      }
    }
  }
}

template <typename T, bool VEC>
__global__ void __launch_bounds__(kThreads, sizeof(T) == 4 ? 4 : 2)
    symv_strip_kernel(long n, long nt, const T *__restrict__ A, long lda, const T *__restrict__ x, T *__restrict__ P,
                      bool upper) {
  constexpr int VN = V16<T>::N;
  constexpr int TPR = kSymTile / VN;       // threads per tile row (16 float, 32 double)
  constexpr int RPP = kThreads / TPR;      // rows per pass
  constexpr int PASSES = kSymTile / RPP;
  __shared__ T colsh[RPP][kSymTile];
  __shared__ T rowpart[kSymTile][TPR + 1];
  __shared__ T diagcol[kSymTile];
  const long strips = ceil_div(nt, long(kSymStrip));
  const long tr = long(blockIdx.x) / strips, s = long(blockIdx.x) % strips;
  // stored tiles of storage tile row tr: lower tc in [0, tr], upper [tr, nt)
  const long t_lo = upper ? tr : 0, t_hi = upper ? nt - 1 : tr;
  const long c0 = t_lo + s * kSymStrip;
  if (c0 > t_hi) return;
  const long c1 = c0 + kSymStrip - 1 < t_hi ? c0 + kSymStrip - 1 : t_hi;
  const int tx = threadIdx.x % TPR, ty = threadIdx.x / TPR;
  const long r0 = tr * kSymTile + ty;
  T xr[PASSES], rowacc[PASSES];
#pragma unroll
  for (int p = 0; p < PASSES; ++p) {
    const long r = r0 + p * RPP;
    xr[p] = r < n ? x[r] : T(0);
    rowacc[p] = T(0);
  }
  if (threadIdx.x < kSymTile) diagcol[threadIdx.x] = T(0);
  T av[PASSES][VN], an[PASSES][VN];
  symv_load<T, VEC, PASSES, VN, RPP>(av, n, r0, c0 * kSymTile + tx * VN, A, lda);
  for (long tc = c0; tc <= c1; ++tc) {
    // next tile's rows in flight while this one is multiplied
    if (tc < c1) symv_load<T, VEC, PASSES, VN, RPP>(an, n, r0, (tc + 1) * kSymTile + tx * VN, A, lda);
    const long c0e = tc * kSymTile + tx * VN;
    T xc[VN], colacc[VN];
#pragma unroll
    for (int e = 0; e < VN; ++e) {
      xc[e] = c0e + e < n ? x[c0e + e] : T(0);
      colacc[e] = T(0);
    }
    const bool diag = tc == tr;
    if (diag)
      symv_tile<true, T, PASSES, VN, RPP>(av, xc, xr, rowacc, colacc, tx * VN, ty, upper);
    else
      symv_tile<false, T, PASSES, VN, RPP>(av, xc, xr, rowacc, colacc, tx * VN, ty, upper);
#pragma unroll
    for (int e = 0; e < VN; ++e) colsh[ty][tx * VN + e] = colacc[e];
    __syncthreads();
    if (threadIdx.x < kSymTile) {
      const int t = threadIdx.x;
      T cs = 0;
#pragma unroll
      for (int q = 0; q < RPP; ++q) cs += colsh[q][t];
      if (diag) {
        diagcol[t] = cs;
      } else {
        const long rcol = tc * kSymTile + t;  // output rows of the tile's columns
        if (rcol < n) P[tr * n + rcol] = cs;
      }
      const long rrow = tr * kSymTile + t;
      if (tc != c0 && rrow < n) P[tc * n + rrow] = T(0);
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PASSES; ++p)
#pragma unroll
      for (int e = 0; e < VN; ++e) av[p][e] = an[p][e];
  }
  // the strip's row sums: per row, the TPR per-thread partials in order
#pragma unroll
  for (int p = 0; p < PASSES; ++p) rowpart[ty + p * RPP][tx] = rowacc[p];
  __syncthreads();
  if (threadIdx.x < kSymTile) {
    const int t = threadIdx.x;
    T rs = 0;
#pragma unroll
    for (int q = 0; q < TPR; ++q) rs += rowpart[t][q];
    const long rrow = tr * kSymTile + t;
    if (rrow < n) P[c0 * n + rrow] = rs + diagcol[t];
  }
}

template <typename T>
void symv(bool upper, long n, T alpha, const T *A, long lda, const T *x, long incx, T beta, T *y, long incy) {
  if (n <= 0) return;
  const long nt = ceil_div(n, kSymTile);
  Carve cv;
  const size_t ox = cv.add<T>(n), op = cv.add<T>(nt * n);
  cv.alloc();
  const T *xu = unit_view(n, x, incx, cv.at<T>(ox));
  T *P = cv.at<T>(op);
  const long grid = nt * ceil_div(nt, long(kSymStrip));
  if (vec_ok(A, lda))
    symv_strip_kernel<T, true><<<unsigned(grid), kThreads, 0, ctx().stream>>>(n, nt, A, lda, xu, P, upper);
  else
    symv_strip_kernel<T, false><<<unsigned(grid), kThreads, 0, ctx().stream>>>(n, nt, A, lda, xu, P, upper);
  EXB_LAUNCH("symv strip kernel");
  count_launch();
  launch_finish<T, 0>(n, int(nt), P, alpha, beta, y, incy, nullptr, false);
}

#define EXB_L2_INST(T)                                                                                   \
  template void gemv<T>(bool, long, long, T, const T *, long, const T *, long, T, T *, long);            \
  template void trmv<T>(bool, bool, bool, long, const T *, long, T *, long);                             \
  template void ger<T>(long, long, T, const T *, long, const T *, long, T *, long);                      \
  template void syr<T>(bool, long, T, const T *, long, T *, long);                                       \
  template void syr2<T>(bool, long, T, const T *, long, const T *, long, T *, long);                     \
  template void symv<T>(bool, long, T, const T *, long, const T *, long, T, T *, long);
EXB_L2_INST(float)
EXB_L2_INST(double)

}  // namespace l2
}  // namespace exb
