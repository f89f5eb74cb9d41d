// Plain-precision level 3 on the CUDA cores: FP32 FFMA (sgemm, ssymm, ssyrk)
// and FP64 DFMA (dgemm, dsymm, dsyrk).  One tiled kernel template, with
// operand loaders that express op(A)/op(B) (gemm), the symmetric operand
// rebuilt from its stored triangle on load (symm) and A A^T / A^T A on the
// triangle's tiles only (syrk).  beta is applied in the epilogue, fused with
// the store, replacing the reference's separate mscal / trmscal pass
// (test/level3/*/exo_*_wrapper.h, src/level3/mscal.py:12-28); it is applied
// as a multiplication even when beta == 0, as that pass does.
// Reference algorithms: src/level3/{gemm,symm,syrk,syr2k,trmm}.py.
#include <cuda_runtime.h>

#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace l3 {

// Operand views: element (r, c) of the logical operand.
template <typename T>
struct Plain {  // op(X) with op = transpose when t
  const T *p;
  long ld;
  bool t;
  __device__ __forceinline__ T operator()(long r, long c) const { return t ? p[c * ld + r] : p[r * ld + c]; }
  __device__ __forceinline__ bool contiguous_cols() const { return !t; }
};
template <typename T>
struct Sym {  // symmetric matrix from its stored triangle
  const T *p;
  long ld;
  bool upper;
  __device__ __forceinline__ T operator()(long r, long c) const {
    const bool stored = upper ? (c >= r) : (c <= r);
    return stored ? p[r * ld + c] : p[c * ld + r];
  }
  __device__ __forceinline__ bool contiguous_cols() const { return true; }
};

template <typename T>
struct Cat {  // [op(X) | op(Y)]: columns c < K from X, the rest from Y (syr2k)
  Plain<T> x, y;
  long K;
  __device__ __forceinline__ T operator()(long r, long c) const { return c < K ? x(r, c) : y(r, c - K); }
  __device__ __forceinline__ bool contiguous_cols() const { return x.contiguous_cols(); }
};
template <typename T, class V>
struct Transposed {  // element (r, c) of V^T
  V v;
  __device__ __forceinline__ T operator()(long r, long c) const { return v(c, r); }
  __device__ __forceinline__ bool contiguous_cols() const { return !v.contiguous_cols(); }
};
template <typename T>
struct Tri {  // op(A) for a triangular A: zero outside the stored triangle, ones on a unit diagonal
  const T *p;
  long ld;
  bool upper, trans, unit;
  __device__ __forceinline__ T operator()(long r, long c) const {
    const long i = trans ? c : r, j = trans ? r : c;  // A's own row / column
    if (i == j) return unit ? T(1) : p[i * ld + i];
    const bool stored = upper ? j > i : j < i;
    return stored ? p[i * ld + j] : T(0);
  }
  __device__ __forceinline__ bool contiguous_cols() const { return !trans; }
};

// Tile configurations: 128x128 (8x8 per thread) for FP32, 64x64 (4x4 per
// thread) for FP64 and for FP32 products too small to give every SM a
// 128x128 tile (sgemm 1024^3 has 64 such tiles for 152 SMs, 256 of 64x64).
template <typename T, bool SMALL = false>
struct Cfg;
template <>
struct Cfg<float, false> {
  static constexpr int BM = 128, BN = 128, BK = 16, TM = 8, TN = 8, THREADS = 256;
};
template <>
struct Cfg<float, true> {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4, THREADS = 256;
};
template <bool SMALL>
struct Cfg<double, SMALL> {
  static constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4, THREADS = 256;
};

// C tile (bm, bn) of rows m x cols n.  mode & 3: 0 all tiles, 1 lower,
// 2 upper (syrk): tiles strictly outside the triangle are not launched and
// elements outside it are left untouched.  mode & 4: C = alpha * acc without
// reading C (trmm overwrites its operand).
template <typename T, class OA, class OB, bool SMALL>
__global__ void __launch_bounds__(Cfg<T, SMALL>::THREADS)
    gemm_kernel(long m, long n, long k, T alpha, OA opA, OB opB, T beta, T *C, long ldc, int mode) {
  using CF = Cfg<T, SMALL>;
  const int tri = mode & 3;
  constexpr int BM = CF::BM, BN = CF::BN, BK = CF::BK, TM = CF::TM, TN = CF::TN;
  constexpr int NT = CF::THREADS;
  constexpr int LA = BM * BK / NT, LB = BN * BK / NT;  // loads per thread per tile
  constexpr int TX = BN / TN;                           // threads along n
  __shared__ T As[2][BK][BM + 4];
  __shared__ T Bs[2][BK][BN + 4];

  long bm, bn;
  if (tri == 0) {
    bm = blockIdx.y;
    bn = blockIdx.x;
  } else {
    // linear index over the lower triangle of tiles (bn <= bm); upper swaps
    const long t = blockIdx.x;
    long r = long((sqrt(8.0 * double(t) + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    const long c = t - r * (r + 1) / 2;
    bm = tri == 1 ? r : c;
    bn = tri == 1 ? c : r;
  }
  const long row0 = bm * BM, col0 = bn * BN;
  const int tid = threadIdx.x;
  const int tx = tid % TX, ty = tid / TX;

  const bool a_kfast = opA.contiguous_cols();  // A(i, k) contiguous along k
  const bool b_nfast = opB.contiguous_cols();  // B(k, j) contiguous along j

  T ra[LA], rb[LB];
  auto fetch = [&](long k0) {
#pragma unroll
    for (int s = 0; s < LA; ++s) {
      const int e = tid + s * NT;
      const int i = a_kfast ? e / BK : e % BM, kk = a_kfast ? e % BK : e / BM;
      const long gi = row0 + i, gk = k0 + kk;
      ra[s] = (gi < m && gk < k) ? opA(gi, gk) : T(0);
    }
#pragma unroll
    for (int s = 0; s < LB; ++s) {
      const int e = tid + s * NT;
      const int j = b_nfast ? e % BN : e / BK, kk = b_nfast ? e / BN : e % BK;
      const long gj = col0 + j, gk = k0 + kk;
      rb[s] = (gj < n && gk < k) ? opB(gk, gj) : T(0);
    }
  };
  auto stash = [&](int buf) {
#pragma unroll
    for (int s = 0; s < LA; ++s) {
      const int e = tid + s * NT;
      const int i = a_kfast ? e / BK : e % BM, kk = a_kfast ? e % BK : e / BM;
      As[buf][kk][i] = ra[s];
    }
#pragma unroll
    for (int s = 0; s < LB; ++s) {
      const int e = tid + s * NT;
      const int j = b_nfast ? e % BN : e / BK, kk = b_nfast ? e / BN : e % BK;
      Bs[buf][kk][j] = rb[s];
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = 0;

  const long ktiles = ceil_div(k, BK);
  if (ktiles > 0) {
    fetch(0);
    stash(0);
  }
  __syncthreads();
  for (long kt = 0; kt < ktiles; ++kt) {
    const int buf = int(kt & 1);
    if (kt + 1 < ktiles) fetch((kt + 1) * BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T av[TM], bv[TN];
      // rows ty*TM/2 .. and BM/2 + ty*TM/2 ..; cols likewise (conflict-free)
#pragma unroll
      for (int a = 0; a < TM / 2; ++a) {
        av[a] = As[buf][kk][ty * (TM / 2) + a];
        av[a + TM / 2] = As[buf][kk][BM / 2 + ty * (TM / 2) + a];
      }
#pragma unroll
      for (int b = 0; b < TN / 2; ++b) {
        bv[b] = Bs[buf][kk][tx * (TN / 2) + b];
        bv[b + TN / 2] = Bs[buf][kk][BN / 2 + tx * (TN / 2) + b];
      }
#pragma unroll
      for (int a = 0; a < TM; ++a)
#pragma unroll
        for (int b = 0; b < TN; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
    }
    if (kt + 1 < ktiles) stash(buf ^ 1);
    __syncthreads();
  }

#pragma unroll
  for (int a = 0; a < TM; ++a) {
    const long gi = row0 + (a < TM / 2 ? ty * (TM / 2) + a : BM / 2 + ty * (TM / 2) + a - TM / 2);
    if (gi >= m) continue;
#pragma unroll
    for (int b = 0; b < TN; ++b) {
      const long gj = col0 + (b < TN / 2 ? tx * (TN / 2) + b : BN / 2 + tx * (TN / 2) + b - TN / 2);
      if (gj >= n) continue;
      if (tri == 1 && gj > gi) continue;
      if (tri == 2 && gj < gi) continue;
      T *c = C + gi * ldc + gj;
      *c = (mode & 4) ? alpha * acc[a][b] : alpha * acc[a][b] + beta * *c;
    }
  }
}

// FP32 fast path for full tiles: 128x128x16, 256 threads with 8x8 results
// each, two CTAs per SM.  Operands come in as 16-byte vectors staged
// through registers (stored transposed into shared memory where op(X) runs
// along k), shared memory is double-buffered, and the inner step reads
// 16-byte vectors of both tiles.  Used when m and n are multiples of 128, k
// of 16, and both operands are 16-byte aligned with leading dimensions that
// are multiples of 4; the generic kernel's per-element operand views take
// 254 registers (one CTA per SM) and scalar loads.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256, 2)
    sgemm_tile_kernel(long m, long n, long k, float alpha, const float *__restrict__ A, long lda,
                      const float *__restrict__ B, long ldb, float beta, float *__restrict__ C, long ldc, int mode) {
  constexpr int BM = 128, BN = 128, BK = 16;
  __shared__ __align__(16) float As[2][BK][BM + 4];
  __shared__ __align__(16) float Bs[2][BK][BN + 4];
  const int tri = mode & 3;
  long bm, bn;
  if (tri == 0) {
    bm = blockIdx.y;
    bn = blockIdx.x;
  } else {
    const long t = blockIdx.x;
    long r = long((sqrt(8.0 * double(t) + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    const long c = t - r * (r + 1) / 2;
    bm = tri == 1 ? r : c;
    bn = tri == 1 ? c : r;
  }
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  // this thread's two 16-byte pieces of each tile: op(A) m x k, op(B) k x n
  //   along k (A not transposed, B transposed): rows/cols r0 = tid/4 and
  //   r0 + 64 of the tile, k offset 4 (tid % 4)
  //   across k (A transposed, B not): k rows tid/32 and tid/32 + 8, offset
  //   4 (tid % 32) along m or n
  const float *pa, *pb;
  long sa, sb;  // element step between the two pieces; step per k tile
  long ka, kb;
  if (!TA) {
    pa = A + (bm * BM + (tid >> 2)) * lda + 4 * (tid & 3);
    sa = 64 * lda;
    ka = BK;
  } else {
    pa = A + long(tid >> 5) * lda + bm * BM + 4 * (tid & 31);
    sa = 8 * lda;
    ka = BK * lda;
  }
  if (TB) {
    pb = B + (bn * BN + (tid >> 2)) * ldb + 4 * (tid & 3);
    sb = 64 * ldb;
    kb = BK;
  } else {
    pb = B + long(tid >> 5) * ldb + bn * BN + 4 * (tid & 31);
    sb = 8 * ldb;
    kb = BK * ldb;
  }
  // the side whose tile is stored as it lies (A transposed, B not) goes
  // straight to shared memory with 16-byte cp.async; the other is staged
  // through registers and stored transposed
  float4 ra[2], rb[2];
  auto fetch = [&](int nbuf) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float *ga = pa + h * sa, *gb = pb + h * sb;
      if (TA) {
        const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(&As[nbuf][(tid >> 5) + 8 * h][4 * (tid & 31)]));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(ga) : "memory");
      } else {
        ra[h] = __ldg(reinterpret_cast<const float4 *>(ga));
      }
      if (!TB) {
        const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(&Bs[nbuf][(tid >> 5) + 8 * h][4 * (tid & 31)]));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gb) : "memory");
      } else {
        rb[h] = __ldg(reinterpret_cast<const float4 *>(gb));
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    pa += ka;
    pb += kb;
  };
  auto stash = [&](int buf) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!TA) {
        const int i = (tid >> 2) + 64 * h, kk = 4 * (tid & 3);
        As[buf][kk][i] = ra[h].x;
        As[buf][kk + 1][i] = ra[h].y;
        As[buf][kk + 2][i] = ra[h].z;
        As[buf][kk + 3][i] = ra[h].w;
      }
      if (TB) {
        const int j = (tid >> 2) + 64 * h, kk = 4 * (tid & 3);
        Bs[buf][kk][j] = rb[h].x;
        Bs[buf][kk + 1][j] = rb[h].y;
        Bs[buf][kk + 2][j] = rb[h].z;
        Bs[buf][kk + 3][j] = rb[h].w;
      }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
  };
  float acc[8][8];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
  const long ktiles = k / BK;
  fetch(0);
  stash(0);
  __syncthreads();
  for (long kt = 0; kt < ktiles; ++kt) {
    const int buf = int(kt & 1);
    // buffer buf ^ 1 was last read before the barrier that ended step kt - 1
    if (kt + 1 < ktiles) fetch(buf ^ 1);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      // rows ty*4 .. +3 and 64 + ty*4 .. +3; columns likewise with tx
      const float4 a0 = *reinterpret_cast<const float4 *>(&As[buf][kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4 *>(&As[buf][kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4 *>(&Bs[buf][kk][64 + tx * 4]);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(av[a], bv[b], acc[a][b]);
    }
    if (kt + 1 < ktiles) stash(buf ^ 1);
    __syncthreads();
  }
  const long row0 = bm * BM, col0 = bn * BN;
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const long gi = row0 + (a < 4 ? ty * 4 + a : 64 + ty * 4 + a - 4);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      const long gj = col0 + (b < 4 ? tx * 4 + b : 64 + tx * 4 + b - 4);
      if (tri == 1 && gj > gi) continue;
      if (tri == 2 && gj < gi) continue;
      float *c = C + gi * ldc + gj;
      *c = alpha * acc[a][b] + beta * *c;
    }
  }
}

// The fast path's conditions (see sgemm_tile_kernel); launches it and
// returns true when they hold.
static bool sgemm_tiles(bool ta, bool tb, long m, long n, long k, float alpha, const float *A, long lda,
                        const float *B, long ldb, float beta, float *C, long ldc, int tri) {
  if (m <= 0 || n <= 0 || k < 16 || m % 128 || n % 128 || k % 16 || lda % 4 || ldb % 4) return false;
  if (!aligned16(A) || !aligned16(B)) return false;
  if (tri && m != n) return false;
  const long tm = m / 128, tn = n / 128;
  if (tri == 0 && tm * tn < ctx().sm_count) return false;  // small products keep the 64x64 tiles
  dim3 grid = tri == 0 ? dim3(unsigned(tn), unsigned(tm)) : dim3(unsigned(tn * (tn + 1) / 2));
  auto kern = ta ? (tb ? sgemm_tile_kernel<true, true> : sgemm_tile_kernel<true, false>)
                 : (tb ? sgemm_tile_kernel<false, true> : sgemm_tile_kernel<false, false>);
  kern<<<grid, 256, 0, ctx().stream>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, tri);
  EXB_LAUNCH("sgemm tile kernel");
  count_launch();
  return true;
}

// The full symmetric matrix S (d x d, row-major, ld = d) from A's stored
// triangle, in 32x32 tiles: the tile and its mirror are read row by row
// (coalesced) into shared memory, and each element of S takes the stored one.
__global__ void __launch_bounds__(256) symmetrize_kernel(long d, const float *__restrict__ A, long lda, bool upper,
                                                         float *__restrict__ S) {
  __shared__ float T1[32][33], T2[32][33];
  const long bi = blockIdx.y, bj = blockIdx.x;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const long i = bi * 32 + r, j = bj * 32 + tx;
    if (i < d && j < d) T1[r][tx] = A[i * lda + j];
    const long i2 = bj * 32 + r, j2 = bi * 32 + tx;
    if (i2 < d && j2 < d) T2[r][tx] = A[i2 * lda + j2];
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const long i = bi * 32 + r, j = bj * 32 + tx;
    if (i >= d || j >= d) continue;
    const bool stored = upper ? (j >= i) : (j <= i);
    S[i * d + j] = stored ? T1[r][tx] : T2[tx][r];
  }
}

template <typename T, bool SMALL, class OA, class OB>
static void launch_cfg(long m, long n, long k, T alpha, OA a, OB b, T beta, T *C, long ldc, int mode) {
  using CF = Cfg<T, SMALL>;
  dim3 grid;
  if ((mode & 3) == 0) {
    grid = dim3(unsigned(ceil_div(n, CF::BN)), unsigned(ceil_div(m, CF::BM)));
  } else {
    const long nt = ceil_div(n, CF::BM);  // BM == BN for every configuration
    grid = dim3(unsigned(nt * (nt + 1) / 2));
  }
  gemm_kernel<T, OA, OB, SMALL><<<grid, CF::THREADS, 0, ctx().stream>>>(m, n, k, alpha, a, b, beta, C, ldc, mode);
  EXB_LAUNCH("gemm kernel");
  count_launch();
}

template <typename T, class OA, class OB>
static void launch(long m, long n, long k, T alpha, OA a, OB b, T beta, T *C, long ldc, int mode) {
  if (m <= 0 || n <= 0) return;
  constexpr int BM = Cfg<T, false>::BM;
  const long tiles = (mode & 3) == 0 ? ceil_div(m, BM) * ceil_div(n, BM) : ceil_div(n, BM) * (ceil_div(n, BM) + 1) / 2;
  if (std::is_same<T, float>::value && tiles < ctx().sm_count)
    launch_cfg<T, true>(m, n, k, alpha, a, b, beta, C, ldc, mode);
  else
    launch_cfg<T, false>(m, n, k, alpha, a, b, beta, C, ldc, mode);
}

// src/level3/gemm.py:17-47 with the wrapper's beta pre-pass fused
template <typename T>
void gemm_simt(bool ta, bool tb, long m, long n, long k, T alpha, const T *A, long lda, const T *B, long ldb, T beta,
               T *C, long ldc) {
  if constexpr (std::is_same<T, float>::value)
    if (sgemm_tiles(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, 0)) return;
  launch<T>(m, n, k, alpha, Plain<T>{A, lda, ta}, Plain<T>{B, ldb, tb}, beta, C, ldc, 0);
}

// src/level3/symm.py:16-47
template <typename T>
void symm_simt(bool left, bool upper, long m, long n, T alpha, const T *A, long lda, const T *B, long ldb, T beta,
               T *C, long ldc) {
  if constexpr (std::is_same<T, float>::value) {
    // full tiles: sym(A) written out once, then the FP32 fast path
    const long d = left ? m : n;
    if (m > 0 && n > 0 && m % 128 == 0 && n % 128 == 0 && ldb % 4 == 0 && aligned16(B) &&
        (m / 128) * (n / 128) >= ctx().sm_count) {
      float *S = static_cast<float *>(scratch(sizeof(float) * size_t(d) * size_t(d)));
      symmetrize_kernel<<<dim3(unsigned(ceil_div(d, 32)), unsigned(ceil_div(d, 32))), 256, 0, ctx().stream>>>(
          d, A, lda, upper, S);
      EXB_LAUNCH("symmetrize kernel");
      count_launch();
      const bool ok = left ? sgemm_tiles(false, false, m, n, m, alpha, S, d, B, ldb, beta, C, ldc, 0)
                           : sgemm_tiles(false, false, m, n, n, alpha, B, ldb, S, d, beta, C, ldc, 0);
      if (ok) return;
    }
  }
  if (left)
    launch<T>(m, n, m, alpha, Sym<T>{A, lda, upper}, Plain<T>{B, ldb, false}, beta, C, ldc, 0);
  else
    launch<T>(m, n, n, alpha, Plain<T>{B, ldb, false}, Sym<T>{A, lda, upper}, beta, C, ldc, 0);
}

// src/level3/syrk.py:17-32: C_tri = alpha * op(A) op(A)^T + beta * C_tri
template <typename T>
void syrk_simt(bool upper, bool trans, long n, long k, T alpha, const T *A, long lda, T beta, T *C, long ldc) {
  // op(A) is n x k: NoTrans A[i,k]; Trans A^T[i,k] = A[k,i].  B = op(A)^T.
  if constexpr (std::is_same<T, float>::value)
    if (sgemm_tiles(trans, !trans, n, n, k, alpha, A, lda, A, lda, beta, C, ldc, upper ? 2 : 1)) return;
  launch<T>(n, n, k, alpha, Plain<T>{A, lda, trans}, Plain<T>{A, lda, !trans}, beta, C, ldc, upper ? 2 : 1);
}

// src/level3/syr2k.py:14-37: C_tri = alpha (op(A) op(B)^T + op(B) op(A)^T)
// + beta C_tri, one product of [op(A) | op(B)] (n x 2k) with [op(B) | op(A)]^T
template <typename T>
void syr2k_simt(bool upper, bool trans, long n, long k, T alpha, const T *A, long lda, const T *B, long ldb, T beta,
                T *C, long ldc) {
  const Cat<T> ab{Plain<T>{A, lda, trans}, Plain<T>{B, ldb, trans}, k};
  const Cat<T> ba{Plain<T>{B, ldb, trans}, Plain<T>{A, lda, trans}, k};
  launch<T>(n, n, 2 * k, alpha, ab, Transposed<T, Cat<T>>{ba}, beta, C, ldc, upper ? 2 : 1);
}

// src/level3/trmm.py:12-78 (Left): B = alpha op(A) B with A triangular
// (right: B = alpha B op(A), used for column-major calls).  B
// is copied to scratch first (the product reads every row of B while it is
// overwritten).  Entries outside the triangle enter the product as zeros, so
// an infinity or NaN in B reaches rows whose triangle excludes it; the
// reference skips those terms.
template <typename T>
void trmm_simt(bool left, bool upper, bool trans, bool unit, long m, long n, T alpha, const T *A, long lda, T *B,
               long ldb) {
  if (m <= 0 || n <= 0) return;
  T *Bc = static_cast<T *>(scratch(sizeof(T) * size_t(m) * size_t(n)));
  EXB_CUDA(cudaMemcpy2DAsync(Bc, sizeof(T) * size_t(n), B, sizeof(T) * size_t(ldb), sizeof(T) * size_t(n), size_t(m),
                             cudaMemcpyDeviceToDevice, ctx().stream));
  if (left)
    launch<T>(m, n, m, alpha, Tri<T>{A, lda, upper, trans, unit}, Plain<T>{Bc, n, false}, T(0), B, ldb, 4);
  else  // B = alpha B op(A), A n x n
    launch<T>(m, n, n, alpha, Plain<T>{Bc, n, false}, Tri<T>{A, lda, upper, trans, unit}, T(0), B, ldb, 4);
}

template void syr2k_simt<float>(bool, bool, long, long, float, const float *, long, const float *, long, float,
                                float *, long);
template void syr2k_simt<double>(bool, bool, long, long, double, const double *, long, const double *, long, double,
                                 double *, long);
template void trmm_simt<float>(bool, bool, bool, bool, long, long, float, const float *, long, float *, long);
template void trmm_simt<double>(bool, bool, bool, bool, long, long, double, const double *, long, double *, long);
template void gemm_simt<float>(bool, bool, long, long, long, float, const float *, long, const float *, long, float,
                               float *, long);
template void gemm_simt<double>(bool, bool, long, long, long, double, const double *, long, const double *, long,
                                double, double *, long);
template void symm_simt<float>(bool, bool, long, long, float, const float *, long, const float *, long, float, float *,
                               long);
template void symm_simt<double>(bool, bool, long, long, double, const double *, long, const double *, long, double,
                                double *, long);
template void syrk_simt<float>(bool, bool, long, long, float, const float *, long, float, float *, long);
template void syrk_simt<double>(bool, bool, long, long, double, const double *, long, double, double *, long);

}  // namespace l3
}  // namespace exb
