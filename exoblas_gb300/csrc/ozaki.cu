// dgemm by Ozaki-style slice emulation on the tcgen05 tensor cores.
//
// Each row i of op(A) is scaled by 2^-e_i and each column j of op(B) by
// 2^-f_j so that every entry is below 1 in magnitude, then written as eight
// balanced base-128 digits with integer arithmetic on the FP64 bit pattern:
//   x 2^-e = sum_{s=0}^{7} a_s 2^{-7(s+1)},  |a_0| <= 128, |a_s| <= 64,
// the low bits beyond 2^-56 rounded away.  The digits are small integers,
// carried exactly in BF16 (8 significand bits).  The digit products of
// weight 2^{-7(d+2)}, d = s + t <= 7 (36 GEMMs), are accumulated per weight d
// in eight FP32 tensor-memory accumulators; with K cut into 256-long chunks
// every accumulator stays an integer below 2^24, so the tensor-core sums are
// exact (per chunk |acc_d| <= 256 (2*128*64 + 6*64*64) < 2^24, and
// |acc_0| <= 256 * 128 * 128).  After each chunk the epilogue warps fold the
// eight integers of every element into two exact int64 sums
//   H = sum_{d<=3} acc_d 2^{7(3-d)},  L = sum_{d>=4} acc_d 2^{7(7-d)},
// and at the end of the tile form, in FP64,
//   C = alpha * 2^{e_i + f_j - 63} (H 2^28 + L) + beta * C.
// (GB300's INT8 tensor path is far slower than its BF16 path, so the
// integer digits ride on BF16 MMAs; the accumulation is exact either way.)
// Dropped products (d >= 8) and the truncated tail weigh below 2^-56 of the
// row/column scale, so the result carries FP64-level componentwise error.
//
// Kernel: one CTA per SM over 128 x 64 tiles; warp 0 TMA (64-byte swizzled
// 32-wide k-blocks of all 8 digit planes of A and of B, 96 KiB per stage,
// 2 stages), warp 1 tcgen05.mma (M = 128, N = 64, K = 16; 72 per k-block),
// warps 2..17 epilogue.  Bounded waits as in gemm_tc.cu.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"
#include "tc5.cuh"

namespace exb {
namespace l3 {
namespace oz {

using namespace tc5;

constexpr int BM = 128, BN = 64, BK = 32;
constexpr int kS = 8;                     // digits per operand
constexpr int kProducts = kS * (kS + 1) / 2;
constexpr int kStages = 2;
constexpr int kATile = BM * BK * 2;       // 8 KiB
constexpr int kBTile = BN * BK * 2;       // 4 KiB
constexpr int kStageBytes = kS * (kATile + kBTile);
constexpr int kChunkKB = 8;               // K = 256 per exact chunk
constexpr int kEpiWarps = 16;
constexpr int kEpiCols = BN / (kEpiWarps / 4);  // 16
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr int kTmemCols = 512;            // accumulator d at column 64 d
constexpr uint32_t kIdesc = idesc_bf16_f32(BM, BN);

__constant__ signed char kPs[kProducts];
__constant__ signed char kPt[kProducts];

struct Params {
  int M, N, K;
  int Mp, Np, kblocks;
  int mtiles, ntiles, tiles;
  int tri;  // 0 full, 1 lower, 2 upper (syrk: only that triangle is written)
  double alpha, beta;
  double *C;
  long ldc;
  const int *ea;  // biased max exponent per row of op(A)
  const int *fb;  // biased max exponent per column of op(B)
  int *status;
};

// tile index -> (mt, nt).  Triangle mode walks the 128 x 128 blocks on and
// below (lower) or above (upper) the diagonal, two 64-wide n-tiles each.
__device__ __forceinline__ void tile_mn(const Params &p, int t, int &mt, int &nt) {
  if (!p.tri) {
    // groups of 8 m-tiles walked along n: the CTAs of one wave share a few
    // A slabs and B slabs, so the digit planes are re-read from L2
    constexpr int G = 8;
    const int group = t / (G * p.ntiles);
    const int first = group * G;
    const int gm = p.mtiles - first < G ? p.mtiles - first : G;
    const int in = t - group * G * p.ntiles;
    mt = first + in % gm;
    nt = in / gm;
    return;
  }
  const int b = t >> 1;
  int r = int((sqrtf(8.f * float(b) + 1.f) - 1.f) * 0.5f);
  while (r * (r + 1) / 2 > b) --r;
  while ((r + 1) * (r + 2) / 2 <= b) ++r;
  const int c = b - r * (r + 1) / 2;
  mt = p.tri == 1 ? r : c;
  nt = 2 * (p.tri == 1 ? c : r) + (t & 1);
}

__global__ void __launch_bounds__(kThreads, 1)
    ozaki_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB, Params p) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], accfull, accempty, drain;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&accfull, 1);
    mbar_init(&accempty, kEpiWarps);
    mbar_init(&drain, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(&tmem_slot, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t round = 0;
      long issued = 0;
      for (int t = blockIdx.x; t < p.tiles && !abort_flag; t += gridDim.x) {
        int mt, nt;
        tile_mn(p, t, mt, nt);
        for (int kb = 0; kb < p.kblocks; ++kb) {
          if (!mbar_wait(&empty[stage], (round & 1) ^ 1, &abort_flag, p.status)) break;
          mbar_expect_tx(&full[stage], kStageBytes);
          unsigned char *st = smem + stage * kStageBytes;
#pragma unroll
          for (int s = 0; s < kS; ++s) {
            tma_load_2d(st + s * kATile, &mapA, &full[stage], kb * BK, s * p.Mp + mt * BM);
            tma_load_2d(st + kS * kATile + s * kBTile, &mapB, &full[stage], kb * BK, s * p.Np + nt * BN);
          }
          ++issued;
          if (++stage == kStages) {
            stage = 0;
            ++round;
          }
        }
      }
      for (int s = 0; s < kStages && issued > 0; ++s) {
        const long uses = issued / kStages + (s < issued % kStages ? 1 : 0);
        if (uses == 0) continue;
        const uint32_t par = uint32_t((uses - 1) & 1);
        const long long t0 = clock64();
        while (!mbar_try_wait(&full[s], par) && clock64() - t0 < kTimeoutCycles) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int stage = 0;
      uint32_t round = 0, chunk = 0;
      bool any = false;
      for (int t = blockIdx.x; t < p.tiles && !abort_flag; t += gridDim.x) {
        for (int kb0 = 0; kb0 < p.kblocks && !abort_flag; kb0 += kChunkKB) {
          if (!mbar_wait(&accempty, (chunk & 1) ^ 1, &abort_flag, p.status)) break;
          tc_fence_after();
          const int kb1 = kb0 + kChunkKB < p.kblocks ? kb0 + kChunkKB : p.kblocks;
          for (int kb = kb0; kb < kb1; ++kb) {
            if (!mbar_wait(&full[stage], round & 1, &abort_flag, p.status)) break;
            tc_fence_after();
            const uint32_t sbase = smem_u32(smem + stage * kStageBytes);
            for (int q = 0; q < kProducts; ++q) {
              const int s = kPs[q], u = kPt[q], d = s + u;
              const uint64_t da = sdesc_sw64(sbase + s * kATile);
              const uint64_t db = sdesc_sw64(sbase + kS * kATile + u * kBTile);
              const bool first = kb == kb0 && s == 0;  // first product of weight d in this chunk
#pragma unroll
              for (int k16 = 0; k16 < BK / 16; ++k16)
                umma(tmem + uint32_t(d * BN), da + uint64_t(2 * k16), db + uint64_t(2 * k16), kIdesc,
                     (first && k16 == 0) ? 0u : 1u);
            }
            umma_commit(&empty[stage]);
            any = true;
            if (++stage == kStages) {
              stage = 0;
              ++round;
            }
          }
          if (abort_flag) break;
          umma_commit(&accfull);
          ++chunk;
        }
      }
      if (any) {
        umma_commit(&drain);
        const long long t0 = clock64();
        while (!mbar_try_wait(&drain, 0) && clock64() - t0 < kTimeoutCycles) {
        }
      }
    }
  } else {
    const int q = warp & 3, part = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    uint32_t chunk = 0;
    for (int t = blockIdx.x; t < p.tiles && !abort_flag; t += gridDim.x) {
      int mt, nt;
      tile_mn(p, t, mt, nt);
      long long H[kEpiCols], L[kEpiCols];
#pragma unroll
      for (int j = 0; j < kEpiCols; ++j) H[j] = L[j] = 0;
      bool ok = true;
      for (int kb0 = 0; kb0 < p.kblocks; kb0 += kChunkKB) {
        if (!mbar_wait(&accfull, chunk & 1, &abort_flag, p.status)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t tb = tmem + (uint32_t(q * 32) << 16) + uint32_t(part * kEpiCols);
#pragma unroll
        for (int d = 0; d < kS; ++d) {
          float v[16];
          tmem_ld16(tb + uint32_t(d * BN), v);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const long long iv = static_cast<long long>(__float2int_rn(v[j]));
            if (d <= 3)
              H[j] += iv << (7 * (3 - d));
            else
              L[j] += iv << (7 * (7 - d));
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&accempty);
        ++chunk;
      }
      if (!ok) break;
      const long gi = long(mt) * BM + row;
      if (gi < p.M) {
        double *crow = p.C + gi * p.ldc;
        const int ei = p.ea[gi] - 1022;
        const long gj0 = long(nt) * BN + part * kEpiCols;
#pragma unroll
        for (int j = 0; j < kEpiCols; ++j) {
          const long gj = gj0 + j;
          if (gj < p.N && !(p.tri == 1 && gj > gi) && !(p.tri == 2 && gj < gi)) {
            const int fj = p.fb[gj] - 1022;
            const double v = scalbn(fma(double(H[j]), 268435456.0, double(L[j])), ei + fj - 63);
            crow[gj] = p.alpha * v + p.beta * crow[gj];
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, kTmemCols);
  }
}

// ------------------------------------------------------- scale and slice --
struct View {  // X(r, k) of the logical rows x K operand
  const double *p;
  long ld;
  bool t;       // element (r, k) at p[k * ld + r]
  int sym = 0;  // 1 / 2: symmetric, only the upper / lower triangle stored
  // columns k >= ks come from a second operand q (same orientation; syr2k)
  const double *q = nullptr;
  long ldq = 0;
  int ks = 1 << 30;
  __device__ double operator()(int r, int k) const {
    if (k >= ks) return t ? q[long(k - ks) * ldq + r] : q[long(r) * ldq + (k - ks)];
    if (sym) {
      const bool direct = sym == 1 ? r <= k : r >= k;
      return direct ? p[long(r) * ld + k] : p[long(k) * ld + r];
    }
    return t ? p[long(k) * ld + r] : p[long(r) * ld + k];
  }
  __device__ bool k_contiguous() const { return sym || !t; }
};

__device__ __forceinline__ int biased_exp(double x) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
  return int((b >> 52) & 0x7FF);
}

// E[r] = max biased exponent of row r (atomicMax over 32 x 32 tiles);
// `bad` is set when a NaN or infinity is present.
__global__ void ozaki_exp_kernel(View X, int rows, int K, int *E, int *bad) {
  __shared__ int tile_max[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool kf = X.k_contiguous();
  for (int i = ty; i < 32; i += 8) {
    const int r = kf ? r0 + i : r0 + tx, k = kf ? k0 + tx : k0 + i;
    int e = 0;
    if (r < rows && k < K) {
      e = biased_exp(X(r, k));
      if (e == 0x7FF) atomicOr(bad, 1);
    }
    if (kf)
      tile_max[i][tx] = e;
    else
      tile_max[tx][i] = e;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int r = r0 + threadIdx.x;
    int m = 0;
    for (int k = 0; k < 32; ++k) m = max(m, tile_max[threadIdx.x][k]);
    if (r < rows && m > 0) atomicMax(E + r, m);
  }
}

// Balanced base-128 digits of X(r, k) * 2^{-(E_r - 1022)} (see the header).
__global__ void ozaki_slice_kernel(View X, int rows, int K, int Rp, int Kp, const int *E, __nv_bfloat16 *out) {
  __shared__ double tile[32][33];
  const int r0 = blockIdx.y * 32, k0 = blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const bool kf = X.k_contiguous();
  for (int i = ty; i < 32; i += 8) {
    const int r = kf ? r0 + i : r0 + tx, k = kf ? k0 + tx : k0 + i;
    const double v = (r < rows && k < K) ? X(r, k) : 0.0;
    if (kf)
      tile[i][tx] = v;
    else
      tile[tx][i] = v;
  }
  __syncthreads();
  const size_t plane = size_t(Rp) * Kp;
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i, k = k0 + tx;
    if (r >= Rp || k >= Kp) continue;
    const double x = tile[i][tx];
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    int bx = int((b >> 52) & 0x7FF);
    long long M = static_cast<long long>(b & ((1ull << 52) - 1));
    if (bx == 0) {
      bx = 1;  // subnormal
    } else {
      M |= 1ll << 52;
    }
    const int emax = r < rows ? max(E[r], 1) : 1;
    // F = |x| * 2^{56 - (emax - 1022)} = M * 2^{bx - emax + 3}
    const int sh = bx - emax + 3;
    long long F;
    if (M == 0)
      F = 0;
    else if (sh >= 0)
      F = M << sh;
    else if (sh > -63)
      F = (M + (1ll << (-sh - 1))) >> (-sh);
    else
      F = 0;
    if (b >> 63) F = -F;
    // digits a_7 .. a_1 in [-64, 63] from the bottom; what remains is a_0,
    // |a_0| <= 128 (exact in BF16)
    float dg[kS];
#pragma unroll
    for (int s = kS - 1; s >= 1; --s) {
      int d = int(F & 127);
      if (d >= 64) d -= 128;
      dg[s] = float(d);
      F = (F - d) >> 7;
    }
    dg[0] = float(F);
    const size_t o = size_t(r) * Kp + k;
#pragma unroll
    for (int s = 0; s < kS; ++s) out[s * plane + o] = __float2bfloat16_rn(dg[s]);
  }
}

static int round_up(long v, int m) { return int((v + m - 1) / m * m); }

static void init_products() {
  static std::once_flag once[64];
  const int dev = ctx().device < 64 ? ctx().device : 63;
  std::call_once(once[dev], [] {
  signed char ps[kProducts], pt[kProducts];
  int q = 0;
  for (int d = 0; d < kS; ++d)
    for (int s = 0; s <= d; ++s) {
      ps[q] = static_cast<signed char>(s);
      pt[q] = static_cast<signed char>(d - s);
      ++q;
    }
  EXB_CUDA(cudaMemcpyToSymbol(kPs, ps, sizeof ps));
  EXB_CUDA(cudaMemcpyToSymbol(kPt, pt, sizeof pt));
  });
}

// Returns false (nothing written) when an input holds NaN or infinity; the
// caller then uses the FP64 FMA kernel, which propagates them.
// C[M, N] = alpha X_A X_B^T + beta C with X_A (M x K) and X_B (N x K).
// tri != 0 (syrk, syr2k): N == M and only that triangle of C is written;
// same_ab (syrk): X_B is X_A, scaled and sliced once.
static bool run(const View &xa, const View &xb, int M, int N, int K, double alpha, double beta, double *C, long ldc,
                int tri, bool same_ab) {
  Context &c = ctx();
  init_products();
  const int Kp = round_up(K, BK * kChunkKB), Mp = round_up(M, BM), Np = tri ? Mp : round_up(N, BN);
  const size_t a_elems = size_t(kS) * Mp * Kp, b_elems = same_ab ? 0 : size_t(kS) * Np * Kp;
  const size_t ebytes = (size_t(Mp + Np + 64) * 4 + 255) & ~size_t(255);
  char *ws = static_cast<char *>(scratch((a_elems + b_elems) * 2 + ebytes + 512));
  __nv_bfloat16 *sa = reinterpret_cast<__nv_bfloat16 *>(ws);
  __nv_bfloat16 *sb = same_ab ? sa : sa + a_elems;
  int *ea = reinterpret_cast<int *>(ws + (a_elems + b_elems) * 2);
  int *fb = same_ab ? ea : ea + Mp;
  int *bad = ea + Mp + Np;
  EXB_CUDA(cudaMemsetAsync(ea, 0, ebytes, c.stream));
  ozaki_exp_kernel<<<dim3(unsigned(ceil_div(K, 32)), unsigned(ceil_div(M, 32))), 256, 0, c.stream>>>(xa, M, K, ea, bad);
  if (!same_ab)
    ozaki_exp_kernel<<<dim3(unsigned(ceil_div(K, 32)), unsigned(ceil_div(N, 32))), 256, 0, c.stream>>>(xb, N, K, fb,
                                                                                                        bad);
  EXB_LAUNCH("ozaki exponent kernel");
  count_launch(same_ab ? 1 : 2);
  int hbad = 0;
  EXB_CUDA(cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, c.stream));
  EXB_CUDA(cudaStreamSynchronize(c.stream));
  if (hbad) return false;
  ozaki_slice_kernel<<<dim3(unsigned(Kp / 32), unsigned(Mp / 32)), 256, 0, c.stream>>>(xa, M, K, Mp, Kp, ea, sa);
  if (!same_ab)
    ozaki_slice_kernel<<<dim3(unsigned(Kp / 32), unsigned(Np / 32)), 256, 0, c.stream>>>(xb, N, K, Np, Kp, fb, sb);
  EXB_LAUNCH("ozaki slice kernel");
  count_launch(same_ab ? 1 : 2);
  const CUtensorMap ma = make_map(sa, long(kS) * Mp, Kp, BK, BM);
  const CUtensorMap mb = make_map(sb, long(kS) * Np, Kp, BK, BN);
  Params p;
  p.M = M;
  p.N = N;
  p.K = K;
  p.Mp = Mp;
  p.Np = Np;
  p.kblocks = Kp / BK;
  p.mtiles = Mp / BM;
  p.ntiles = Np / BN;
  p.tri = tri;
  p.tiles = tri ? p.mtiles * (p.mtiles + 1) : p.mtiles * p.ntiles;
  p.alpha = alpha;
  p.beta = beta;
  p.C = C;
  p.ldc = ldc;
  p.ea = ea;
  p.fb = fb;
  p.status = device_status_word();
  static std::once_flag attr[64];
  const int smem = kStages * kStageBytes + 1024;
  const int dev = c.device < 64 ? c.device : 63;
  std::call_once(attr[dev], [smem] {
    EXB_CUDA(cudaFuncSetAttribute(ozaki_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  });
  const int grid = p.tiles < c.sm_count ? p.tiles : c.sm_count;
  ozaki_gemm_kernel<<<grid, kThreads, smem, c.stream>>>(ma, mb, p);
  EXB_LAUNCH("ozaki tcgen05 gemm kernel");
  count_launch();
  c.status_pending = true;
  return true;
}

}  // namespace oz

bool dgemm_ozaki(bool ta, bool tb, long m, long n, long k, double alpha, const double *A, long lda, const double *B,
                 long ldb, double beta, double *C, long ldc) {
  if (m <= 0 || n <= 0 || k <= 0) return false;
  // X_A = op(A); X_B(j, k) = op(B)[k][j]
  return oz::run(oz::View{A, lda, ta}, oz::View{B, ldb, !tb}, int(m), int(n), int(k), alpha, beta, C, ldc, 0, false);
}

// C_tri = alpha op(A) op(A)^T + beta C_tri over the stored triangle only
// (syrk; op(A) = A for NoTrans, A^T for Trans).
bool dsyrk_ozaki(bool upper, bool trans, long n, long k, double alpha, const double *A, long lda, double beta,
                 double *C, long ldc) {
  if (n <= 0 || k <= 0) return false;
  const oz::View x{A, lda, trans};
  return oz::run(x, x, int(n), int(n), int(k), alpha, beta, C, ldc, upper ? 2 : 1, true);
}

// C_tri = alpha (op(A) op(B)^T + op(B) op(A)^T) + beta C_tri (syr2k) as the
// triangle of [op(A) | op(B)] [op(B) | op(A)]^T
bool dsyr2k_ozaki(bool upper, bool trans, long n, long k, double alpha, const double *A, long lda, const double *B,
                  long ldb, double beta, double *C, long ldc) {
  if (n <= 0 || k <= 0) return false;
  const oz::View ab{A, lda, trans, 0, B, ldb, int(k)}, ba{B, ldb, trans, 0, A, lda, int(k)};
  return oz::run(ab, ba, int(n), int(n), int(2 * k), alpha, beta, C, ldc, upper ? 2 : 1, false);
}

// C = alpha sym(A) B + beta C (left) or alpha B sym(A) + beta C (right),
// sym(A) read from its stored triangle.
bool dsymm_ozaki(bool left, bool upper, long m, long n, double alpha, const double *A, long lda, const double *B,
                 long ldb, double beta, double *C, long ldc) {
  if (m <= 0 || n <= 0) return false;
  const oz::View sa{A, lda, false, upper ? 1 : 2};
  if (left) return oz::run(sa, oz::View{B, ldb, true}, int(m), int(n), int(m), alpha, beta, C, ldc, 0, false);
  return oz::run(oz::View{B, ldb, false}, sa, int(m), int(n), int(n), alpha, beta, C, ldc, 0, false);
}

}  // namespace l3
}  // namespace exb
