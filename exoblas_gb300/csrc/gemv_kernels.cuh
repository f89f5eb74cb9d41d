// Device kernels of the gemv family (row dots, column sums, partial-sum
// finish, strided-vector pack), shared by the level-2 launchers and the
// allocation-free sgemv entry point.
#pragma once

#include "common.cuh"

namespace exb {
namespace l2 {

constexpr int kThreads = 256;

// Contiguous copy of a strided vector (element i of src at src[i*inc]);
// 16-byte vectors when the copy is unit-stride and both ends are aligned.
template <typename T>
__global__ void pack_kernel(long n, const T *__restrict__ src, long inc, T *__restrict__ dst) {
  const long stride = long(gridDim.x) * blockDim.x, t = long(blockIdx.x) * blockDim.x + threadIdx.x;
  if (inc == 1 && ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
    using V = typename V16<T>::type;
    constexpr int VN = V16<T>::N;
    const long nv = n / VN;
    const V *s = reinterpret_cast<const V *>(src);
    V *d = reinterpret_cast<V *>(dst);
    for (long i = t; i < nv; i += stride) d[i] = ld_stream(s + i);
    for (long i = nv * VN + t; i < n; i += stride) dst[i] = src[i];
    return;
  }
  for (long i = t; i < n; i += stride) dst[i] = src[i * inc];
}
// ------------------------------------------------------------ row dots ----
// out_i = sum_{j in [lo(i), hi(i))} A[i,j] * x[j] for every row i, G threads
// per row.  MODE 0 (gemv N): y_i = alpha*dot + beta*y_i.  MODE 1 (trmv N):
// x_i = dot (+ xs_i for a unit diagonal, the diagonal being excluded from
// the range).  `tri`: 0 full row, 1 lower (j <= i), 2 upper (j >= i).
template <typename T, int G, bool VEC, int MODE>
__global__ void __launch_bounds__(kThreads)
    rowdot_kernel(long rows, long cols, T alpha, const T *__restrict__ A, long lda, const T *__restrict__ x, T beta,
                  T *y, long incy, int tri, bool unit) {
  using V = typename V16<T>::type;
  constexpr int VN = V16<T>::N;
  constexpr int RPW = 32 / G;  // rows per warp
  const int lane = threadIdx.x & 31;
  const int sub = lane % G;
  const long warp_global = (long(blockIdx.x) * kThreads + threadIdx.x) / 32;
  const long nwarps = long(gridDim.x) * (kThreads / 32);
  long pass = 0;
  for (long base = warp_global * RPW; base < rows; base += nwarps * RPW, ++pass) {
    long i = base + lane / G;
    if (tri != 0 && (pass & 1)) {
      // triangle rows snake: odd passes over the rows run mirrored, so a
      // warp's short and long rows pair up and every warp gets equal work
      const long cs = pass * nwarps * RPW;
      const long ce = cs + nwarps * RPW < rows ? cs + nwarps * RPW : rows;
      i = i < ce ? ce - 1 - (i - cs) : rows;
    }
    T acc = 0;
    if (i < rows) {
      long lo = 0, hi = cols;
      if (tri == 1) hi = (unit ? i : i + 1);
      else if (tri == 2) lo = (unit ? i + 1 : i);
      if (hi > cols) hi = cols;
      const T *a = A + i * lda;
      if (VEC && hi - lo >= VN) {
        // scalar head up to a 16-byte boundary, then vectors, then a scalar tail
        const long vlo = (lo + VN - 1) / VN * VN, vhi = hi / VN * VN;
        for (long j = lo + sub; j < vlo && j < hi; j += G) acc = fma(a[j], x[j], acc);
        const V *av = reinterpret_cast<const V *>(a);
        const V *xv = reinterpret_cast<const V *>(x);
        long v = vlo / VN + sub;
        const long ve = vhi / VN;
        // software pipeline: the row's next 4 vectors are loaded before the
        // current 4 are consumed (x comes from L1/L2 at use).  Two register
        // buffers alternate (the body is written twice), so no vector is
        // copied between registers; measured faster than copying the
        // prefetched buffer (sgemv N 0.93 -> 0.99 of the HBM copy bandwidth).
        V r0[4], r1[4];
        auto load = [&](V(&buf)[4], long at) {
#pragma unroll
          for (int u = 0; u < 4; ++u) buf[u] = ld_stream(av + at + u * G);
        };
        auto use = [&](V(&buf)[4], long at) {
          V xr[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) xr[u] = xv[at + u * G];
#pragma unroll
          for (int e = 0; e < VN; ++e)
#pragma unroll
            for (int u = 0; u < 4; ++u) acc = fma(vget<T>(buf[u], e), vget<T>(xr[u], e), acc);
        };
        bool have = v + 3 * G < ve;
        if (have) load(r0, v);
        while (have) {
          long vn = v + 4 * G;
          bool more = vn + 3 * G < ve;
          if (more) load(r1, vn);
          use(r0, v);
          v = vn;
          if (!more) break;
          vn = v + 4 * G;
          more = vn + 3 * G < ve;
          if (more) load(r0, vn);
          use(r1, v);
          v = vn;
          have = more;
        }
        for (; v < ve; v += G) {
          V a0 = ld_stream(av + v), x0 = xv[v];
#pragma unroll
          for (int e = 0; e < VN; ++e) acc = fma(vget<T>(a0, e), vget<T>(x0, e), acc);
        }
        for (long j = (vhi > vlo ? vhi : vlo) + sub; j < hi; j += G) acc = fma(a[j], x[j], acc);
      } else {
        for (long j = lo + sub; j < hi; j += G) acc = fma(a[j], x[j], acc);
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (i < rows && sub == 0) {
      if (MODE == 0) {
        T *yi = y + i * incy;
        *yi = alpha * acc + beta * *yi;
      } else {
        y[i * incy] = unit ? acc + x[i] : acc;
      }
    }
  }
}

// ------------------------------------------------------------ column sums --
// partial[c][j] = sum over rows i of chunk c of A[i,j] * x[i] (restricted to
// the triangle when tri != 0).  A warp covers 32*VN columns; the 8 warps of
// a CTA take interleaved rows of the chunk and are summed in warp order.
template <typename T, bool VEC>
__global__ void __launch_bounds__(kThreads)
    colsum_kernel(long rows, long cols, const T *__restrict__ A, long lda, const T *__restrict__ x, long rows_per_chunk,
                  T *__restrict__ partial, int tri, bool unit) {
  using V = typename V16<T>::type;
  constexpr int VN = V16<T>::N;
  __shared__ T sh[kThreads / 32][32 * VN];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long j0 = long(blockIdx.x) * 32 * VN + lane * VN;
  const long r0 = long(blockIdx.y) * rows_per_chunk;
  long r1 = r0 + rows_per_chunk;
  if (r1 > rows) r1 = rows;
  T acc[VN];
#pragma unroll
  for (int e = 0; e < VN; ++e) acc[e] = 0;
  // rows of the triangle that can touch columns [j0, j0+VN)
  long rlo = r0, rhi = r1;
  if (tri == 1 && rlo < j0) rlo = j0;                       // lower: i >= j
  if (tri == 2 && rhi > j0 + VN) rhi = j0 + VN;             // upper: i <= j
  const bool full_vec = VEC && j0 + VN <= cols;
  long i = rlo + warp;
  if (full_vec && tri == 0) {
    for (; i + 3 * 8 < rhi; i += 4 * 8) {
      V a0 = ld_stream(reinterpret_cast<const V *>(A + i * lda + j0));
      V a1 = ld_stream(reinterpret_cast<const V *>(A + (i + 8) * lda + j0));
      V a2 = ld_stream(reinterpret_cast<const V *>(A + (i + 16) * lda + j0));
      V a3 = ld_stream(reinterpret_cast<const V *>(A + (i + 24) * lda + j0));
      const T x0 = x[i], x1 = x[i + 8], x2 = x[i + 16], x3 = x[i + 24];
#pragma unroll
      for (int e = 0; e < VN; ++e) {
        acc[e] = fma(vget<T>(a0, e), x0, acc[e]);
        acc[e] = fma(vget<T>(a1, e), x1, acc[e]);
        acc[e] = fma(vget<T>(a2, e), x2, acc[e]);
        acc[e] = fma(vget<T>(a3, e), x3, acc[e]);
      }
    }
  }
  for (; i < rhi; i += 8) {
    const T xi = x[i];
    if (full_vec) {
      V a = ld_stream(reinterpret_cast<const V *>(A + i * lda + j0));
#pragma unroll
      for (int e = 0; e < VN; ++e) {
        const long j = j0 + e;
        const bool in = tri == 0 || (tri == 1 ? (unit ? j < i : j <= i) : (unit ? j > i : j >= i));
        if (in) acc[e] = fma(vget<T>(a, e), xi, acc[e]);
      }
    } else {
#pragma unroll
      for (int e = 0; e < VN; ++e) {
        const long j = j0 + e;
        if (j >= cols) continue;
        const bool in = tri == 0 || (tri == 1 ? (unit ? j < i : j <= i) : (unit ? j > i : j >= i));
        if (in) acc[e] = fma(A[i * lda + j], xi, acc[e]);
      }
    }
  }
#pragma unroll
  for (int e = 0; e < VN; ++e) sh[warp][lane * VN + e] = acc[e];
  __syncthreads();
  for (int t = threadIdx.x; t < 32 * VN; t += kThreads) {
    T s = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w) s += sh[w][t];
    const long j = long(blockIdx.x) * 32 * VN + t;
    if (j < cols) partial[long(blockIdx.y) * cols + j] = s;
  }
}

// MODE 0: y_j = alpha * sum_c partial[c][j] + beta * y_j (gemv T, symv)
// MODE 1: y_j = sum_c partial[c][j] (+ xs_j when unit)  (trmv T)
// A CTA (kThreads) takes 32 consecutive j at a time: warp w sums slots
// [w*chunks/8, (w+1)*chunks/8) in order, and the 8 warp sums are added in
// warp order, so the result depends only on `chunks`.
constexpr int kFinishCols = 32;
template <typename T, int MODE>
__global__ void __launch_bounds__(kThreads)
    finish_kernel(long cols, int chunks, const T *__restrict__ partial, T alpha, T beta, T *y, long incy,
                  const T *xs, bool unit) {
  constexpr int kW = kThreads / 32;
  __shared__ T sh[kW][kFinishCols];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c0 = int(long(chunks) * w / kW), c1 = int(long(chunks) * (w + 1) / kW);
  for (long g = blockIdx.x; g * kFinishCols < cols; g += gridDim.x) {
    const long j = g * kFinishCols + lane;
    T s = 0;
    if (j < cols) {
      int c = c0;
      for (; c + 3 < c1; c += 4) {
        const T p0 = partial[long(c) * cols + j], p1 = partial[long(c + 1) * cols + j],
                p2 = partial[long(c + 2) * cols + j], p3 = partial[long(c + 3) * cols + j];
        s += p0;
        s += p1;
        s += p2;
        s += p3;
      }
      for (; c < c1; ++c) s += partial[long(c) * cols + j];
    }
    sh[w][lane] = s;
    __syncthreads();
    if (w == 0 && j < cols) {
      T t = 0;
#pragma unroll
      for (int q = 0; q < kW; ++q) t += sh[q][lane];
      T *yj = y + j * incy;
      if (MODE == 0)
        *yj = alpha * t + beta * *yj;
      else
        *yj = unit ? t + xs[j] : t;
    }
    __syncthreads();
  }
}

// CTAs for finish_kernel over `cols` outputs, at most `cap`
inline long finish_blocks(long cols, long cap) {
  long b = (cols + kFinishCols - 1) / kFinishCols;
  if (b > cap) b = cap;
  return b < 1 ? 1 : b;
}

}  // namespace l2
}  // namespace exb
