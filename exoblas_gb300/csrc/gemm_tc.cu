// Level 3 on the 5th-generation tensor cores (tcgen05, sm_103a): FP32
// sgemm / ssymm / ssyrk through a split-BF16 representation.
//
// Each FP32 operand x is split into three BF16 terms x = x0 + x1 + x2
// (x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1)), 24 significand
// bits in all.  C = alpha * op(A) op(B) + beta * C is formed from the six
// products whose weight is at least 2^-16 relative to the leading one,
// issued from small to large:
//   lo += a2 b0 + a1 b1 + a0 b2 + a1 b0 + a0 b1,   hi += a0 b0,
// both accumulated in FP32 in tensor memory.  Every bf16 x bf16 product is
// exact in FP32; keeping the leading term in its own accumulator keeps the
// small corrections from being absorbed by it.  The tensor core's FP32
// accumulation does not round to nearest at every step, so K is cut into
// chunks of kChunk: each chunk is accumulated in tensor memory (two buffers,
// alternating), and the epilogue warps fold every finished chunk into
// per-element FP32 sums carried with a TwoSum compensation term, then form
// alpha * sum + beta * C once at the end of the tile.
//
// Kernel structure (one CTA per SM, persistent over 128 x 128 output tiles):
//   warp 0       TMA producer: per k-block, the 3 slices of A and of B (six
//                16 KiB 128-byte-swizzled tiles, one 96 KiB stage, 2 stages)
//   warp 1       allocates tensor memory; one thread issues tcgen05.mma
//                (M = 128, N = 128, K = 16) and tcgen05.commit
//   warps 2..17  epilogue: per chunk, tcgen05.ld of both accumulators of a
//                buffer (four warps per 32-lane quarter, 32 columns each);
//                per tile, beta * C fused into the store, C accessed in
//                32-byte row segments through shared memory (syrk: elements
//                outside the triangle are left alone)
// Synchronisation is by mbarriers; every wait is bounded by a clock budget
// after which the CTA records a timeout in the device status word, drains
// what it started and frees its tensor memory.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"
#include "tc5.cuh"

namespace exb {
namespace l3 {
namespace t5 {

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int kSlices = 3;
constexpr int kStages = 2;
constexpr int kTileBytes = BM * BK * 2;  // 16 KiB (BN == BM)
constexpr int kStageBytes = 2 * kSlices * kTileBytes;
constexpr int kEpiWarps = 16;
constexpr int kEpiCols = BN / (kEpiWarps / 4);  // columns per epilogue warp
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr int kChunkKB = 4;      // k-blocks per accumulation chunk (K = 256)
constexpr int kEpiSmem = kEpiWarps * 32 * 9 * 4;  // per epilogue warp: 32 rows x 8 columns, row pitch 9
constexpr int kDynSmem = kStages * kStageBytes + 1024 + kEpiSmem;
constexpr int kTmemCols = 512;   // two buffers x (hi at column 0, lo at BN)

// products in issue order (small to large); acc 1 = lo, 0 = hi
__constant__ signed char kProdA[6] = {2, 1, 0, 1, 0, 0};
__constant__ signed char kProdB[6] = {0, 1, 2, 0, 1, 0};
__constant__ signed char kProdAcc[6] = {1, 1, 1, 1, 1, 0};

struct Params {
  int M, N, K;
  int Mp, Np;  // slice row pitch (multiples of 128)
  int kblocks;
  int mtiles, ntiles, tiles;
  int tri;  // 0 full, 1 lower, 2 upper (syrk)
  float alpha, beta;
  float *C;
  long ldc;
  int *status;
};

constexpr uint32_t kIdesc = tc5::idesc_bf16_f32(BM, BN);
using namespace tc5;

// tile index -> (mt, nt); grouped raster of 8 m-tiles for L2 reuse; triangle
// tiles for syrk (lower: nt <= mt, upper: nt >= mt)
__device__ __forceinline__ void tile_coords(const Params &p, int t, int &mt, int &nt) {
  if (p.tri) {
    int r = int((sqrtf(8.f * float(t) + 1.f) - 1.f) * 0.5f);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    const int c = t - r * (r + 1) / 2;
    mt = p.tri == 1 ? r : c;
    nt = p.tri == 1 ? c : r;
    return;
  }
  constexpr int G = 8;
  const int group = t / (G * p.ntiles);
  const int first = group * G;
  const int gm = p.mtiles - first < G ? p.mtiles - first : G;
  const int in = t - group * G * p.ntiles;
  mt = first + in % gm;
  nt = in / gm;
}

// A group of independent products for split_bf16_group_kernel: per
// product its two tensor maps (slice planes) and epilogue parameters; per
// output tile an item (product, m-tile, n-tile).
struct alignas(128) TcGroupGemm {
  CUtensorMap ma, mb;
  int M, N, Mp, Np, kblocks;
  float alpha, beta;
  float *C;
  long ldc;
};
struct TcItem {
  int g, mt, nt, pad;
};

// What each role needs to know about output tile t of its sequence: the
// operands' tensor maps and slice pitches, the tile's origin, its k-blocks
// and the epilogue's parameters.
struct TileRef {
  const CUtensorMap *ma, *mb;
  int Mp, Np;      // slice row pitches of the two planes
  int am, bn;      // tile origin: rows am.. of op(A), columns bn.. of op(B)
  int kblocks;
  int M, N, tri;
  float alpha, beta;
  float *C;
  long ldc;
};

// One product (split_bf16_gemm_kernel): tiles in grouped raster order.
struct SingleSrc {
  const CUtensorMap *ma, *mb;
  const Params *p;
  __device__ __forceinline__ void tile(int t, TileRef &r) const {
    int mt, nt;
    tile_coords(*p, t, mt, nt);
    r.ma = ma;
    r.mb = mb;
    r.Mp = p->Mp;
    r.Np = p->Np;
    r.am = mt * BM;
    r.bn = nt * BN;
    r.kblocks = p->kblocks;
    r.M = p->M;
    r.N = p->N;
    r.tri = p->tri;
    r.alpha = p->alpha;
    r.beta = p->beta;
    r.C = p->C;
    r.ldc = p->ldc;
  }
};

// A group of independent products (split_bf16_group_kernel): each item is
// one output tile of one product, items longest first.
struct GroupSrc {
  const TcGroupGemm *gg;
  const TcItem *items;
  __device__ __forceinline__ void tile(int t, TileRef &r) const {
    const TcItem it = items[t];
    const TcGroupGemm &g = gg[it.g];
    r.ma = &g.ma;
    r.mb = &g.mb;
    r.Mp = g.Mp;
    r.Np = g.Np;
    r.am = it.mt * BM;
    r.bn = it.nt * BN;
    r.kblocks = g.kblocks;
    r.M = g.M;
    r.N = g.N;
    r.tri = 0;
    r.alpha = g.alpha;
    r.beta = g.beta;
    r.C = g.C;
    r.ldc = g.ldc;
  }
};

// ------------------------------------------------------------------ body --
// The persistent tile loop shared by both kernels: tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... of the source's ntiles.
template <class Src>
__device__ __forceinline__ void tc_body(const Src &src, int ntiles, int *status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned stage area (128B-swizzle atoms need it)
  unsigned char *smem = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], accfull[2], accempty[2], drain;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], kEpiWarps);  // one arrival per epilogue warp
    }
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
    // ------------------------------------------------------ TMA producer --
    if (lane == 0) {
      int stage = 0;
      uint32_t round = 0;
      long issued = 0;
      const CUtensorMap *last_ma = nullptr;
      for (int t = blockIdx.x; t < ntiles && !abort_flag; t += gridDim.x) {
        TileRef r;
        src.tile(t, r);
        if (r.ma != last_ma) {
          asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(r.ma)) : "memory");
          asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(r.mb)) : "memory");
          last_ma = r.ma;
        }
        for (int kb = 0; kb < r.kblocks; ++kb) {
          if (!mbar_wait(&empty[stage], (round & 1) ^ 1, &abort_flag, status)) break;
          mbar_expect_tx(&full[stage], kStageBytes);
          unsigned char *st = smem + stage * kStageBytes;
#pragma unroll
          for (int s = 0; s < kSlices; ++s) {
            tma_load_2d(st + s * kTileBytes, r.ma, &full[stage], kb * BK, s * r.Mp + r.am);
            tma_load_2d(st + (kSlices + s) * kTileBytes, r.mb, &full[stage], kb * BK, s * r.Np + r.bn);
          }
          ++issued;
          if (++stage == kStages) {
            stage = 0;
            ++round;
          }
        }
      }
      // drain: every issued stage's copies must land before the CTA exits
      for (int s = 0; s < kStages && issued > 0; ++s) {
        // the most recent use of each stage is round r_s; wait for its fill
        long uses = issued / kStages + (s < issued % kStages ? 1 : 0);
        if (uses == 0) continue;
        const uint32_t par = uint32_t((uses - 1) & 1);
        const long long t0 = clock64();
        while (!mbar_try_wait(&full[s], par) && clock64() - t0 < kTimeoutCycles) {
        }
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------- MMA issuer --
    if (lane == 0) {
      int stage = 0;
      uint32_t round = 0;
      uint32_t chunk = 0;  // global chunk counter: buffer chunk & 1
      bool any = false;
      for (int t = blockIdx.x; t < ntiles && !abort_flag; t += gridDim.x) {
        TileRef r;
        src.tile(t, r);
        for (int kb0 = 0; kb0 < r.kblocks && !abort_flag; kb0 += kChunkKB) {
          const int buf = int(chunk & 1);
          if (!mbar_wait(&accempty[buf], ((chunk >> 1) & 1) ^ 1, &abort_flag, status)) break;
          tc_fence_after();
          const uint32_t accbase = tmem + uint32_t(buf * 2 * BN);
          const int kb1 = kb0 + kChunkKB < r.kblocks ? kb0 + kChunkKB : r.kblocks;
          for (int kb = kb0; kb < kb1; ++kb) {
            if (!mbar_wait(&full[stage], round & 1, &abort_flag, status)) break;
            tc_fence_after();
            const uint32_t sbase = smem_u32(smem + stage * kStageBytes);
#pragma unroll
            for (int q = 0; q < 6; ++q) {
              const uint32_t acc = accbase + (kProdAcc[q] ? BN : 0);
              const uint64_t da = sdesc_sw128(sbase + kProdA[q] * kTileBytes);
              const uint64_t db = sdesc_sw128(sbase + (kSlices + kProdB[q]) * kTileBytes);
              // the first product into each accumulator of a chunk overwrites it
              const bool first = kb == kb0 && (q == 0 || q == 5);
#pragma unroll
              for (int k16 = 0; k16 < BK / 16; ++k16)
                umma(acc, da + uint64_t(2 * k16), db + uint64_t(2 * k16), kIdesc, (first && k16 == 0) ? 0u : 1u);
            }
            umma_commit(&empty[stage]);  // frees the stage when these MMAs finish
            any = true;
            if (++stage == kStages) {
              stage = 0;
              ++round;
            }
          }
          if (abort_flag) break;
          umma_commit(&accfull[buf]);
          ++chunk;
        }
      }
      // drain outstanding MMAs before tensor memory is released
      if (any) {
        umma_commit(&drain);
        const long long t0 = clock64();
        while (!mbar_try_wait(&drain, 0) && clock64() - t0 < kTimeoutCycles) {
        }
      }
    }
  } else {
    // --------------------------------------------------------- epilogue --
    const int q = warp & 3;                 // tensor-memory lane quarter this warp may read
    const int part = (warp - 2) >> 2;       // columns [kEpiCols part, kEpiCols (part + 1))
    const int row = q * 32 + lane;
    uint32_t chunk = 0;
    for (int t = blockIdx.x; t < ntiles && !abort_flag; t += gridDim.x) {
      TileRef r;
      src.tile(t, r);
      float sum[kEpiCols], comp[kEpiCols];
#pragma unroll
      for (int j = 0; j < kEpiCols; ++j) sum[j] = comp[j] = 0.f;
      bool ok = true;
      for (int kb0 = 0; kb0 < r.kblocks; kb0 += kChunkKB) {
        const int buf = int(chunk & 1);
        if (!mbar_wait(&accfull[buf], (chunk >> 1) & 1, &abort_flag, status)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t tb = tmem + (uint32_t(q * 32) << 16) + uint32_t(buf * 2 * BN + part * kEpiCols);
#pragma unroll
        for (int c = 0; c < kEpiCols; c += 8) {
          float hi[8], lo[8];
          tmem_ld8(tb + c, hi);
          tmem_ld8(tb + BN + c, lo);
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            // TwoSum of the running sum and this chunk's value
            const float v = hi[j] + lo[j];
            const float s1 = sum[c + j] + v;
            const float z = s1 - sum[c + j];
            comp[c + j] += (sum[c + j] - (s1 - z)) + (v - z);
            sum[c + j] = s1;
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&accempty[buf]);
        ++chunk;
      }
      if (!ok) break;
      // C is read and written through shared memory in 32-byte row segments:
      // per 8 columns, lane `row` stores alpha * sum of its 8 elements, then
      // lane l takes row 4i + l/8, column l%8 (i = 0..7).  (A lane per row
      // touched 32 lines per warp access: 31 sectors per request.)
      float *cs = reinterpret_cast<float *>(smem + kStages * kStageBytes) + (warp - 2) * (32 * 9);
      const long grow0 = long(r.am) + q * 32, gcol0 = long(r.bn) + part * kEpiCols;
#pragma unroll
      for (int c8 = 0; c8 < kEpiCols; c8 += 8) {
#pragma unroll
        for (int j = 0; j < 8; ++j) cs[lane * 9 + j] = r.alpha * (sum[c8 + j] + comp[c8 + j]);
        __syncwarp();
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int rr = 4 * i + (lane >> 3), cc = lane & 7;
          const long gi = grow0 + rr, gj = gcol0 + c8 + cc;
          const bool in = gi < r.M && gj < r.N && !(r.tri == 1 && gj > gi) && !(r.tri == 2 && gj < gi);
          if (in) {
            float *cp = r.C + gi * r.ldc + gj;
            *cp = cs[rr * 9 + cc] + r.beta * *cp;
          }
        }
        __syncwarp();
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

// ---------------------------------------------------------------- kernels --
__global__ void __launch_bounds__(kThreads, 1)
    split_bf16_gemm_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                           Params p) {
  const SingleSrc src{&mapA, &mapB, &p};
  tc_body(src, p.tiles, p.status);
}

__global__ void __launch_bounds__(kThreads, 1)
    split_bf16_group_kernel(const TcGroupGemm *__restrict__ gg, const TcItem *__restrict__ items, int nitems,
                            int *status) {
  const GroupSrc src{gg, items};
  tc_body(src, nitems, status);
}

// --------------------------------------------------------------- split ----
// out[s][r][k] (s < 3, r < Rp, k < Kp, bf16) for the logical rows x K operand
// X(r, k); zero outside rows x K.  32 x 32 tiles through shared memory so
// both the source (either orientation) and the K-major output are coalesced.
template <class Op>
__device__ __forceinline__ void split3_tile(const Op &X, int rows, int K, int Rp, int Kp, __nv_bfloat16 *out, int r0,
                                            int k0) {
  __shared__ float tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  const bool src_k_fast = X.k_contiguous();
  for (int i = ty; i < 32; i += 8) {
    // source read: consecutive threads along the source's contiguous index
    const int r = src_k_fast ? r0 + i : r0 + tx;
    const int k = src_k_fast ? k0 + tx : k0 + i;
    float v = (r < rows && k < K) ? X(r, k) : 0.f;
    if (src_k_fast)
      tile[i][tx] = v;
    else
      tile[tx][i] = v;
  }
  __syncthreads();
  const size_t slice = size_t(Rp) * Kp;
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i, k = k0 + tx;
    if (r >= Rp || k >= Kp) continue;
    const float v = tile[i][tx];
    const __nv_bfloat16 b0 = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(b0);
    const __nv_bfloat16 b1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(b1);
    const __nv_bfloat16 b2 = __float2bfloat16_rn(r2);
    const size_t o = size_t(r) * Kp + k;
    out[o] = b0;
    out[slice + o] = b1;
    out[2 * slice + o] = b2;
  }
}

template <class Op>
__global__ void split3_kernel(Op X, int rows, int K, int Rp, int Kp, __nv_bfloat16 *out) {
  split3_tile(X, rows, K, Rp, Kp, out, int(blockIdx.y) * 32, int(blockIdx.x) * 32);
}

// operand views: X(r, k) for the logical rows x K operand
struct ViewPlain {
  const float *p;
  long ld;
  bool t;  // element (r, k) at p[k * ld + r]
  __device__ float operator()(int r, int k) const { return t ? p[long(k) * ld + r] : p[long(r) * ld + k]; }
  __device__ bool k_contiguous() const { return !t; }
};
struct ViewCat {  // [X | Y]: k < K from X, the rest from Y (syr2k)
  ViewPlain x, y;
  int K;
  __device__ float operator()(int r, int k) const { return k < K ? x(r, k) : y(r, k - K); }
  __device__ bool k_contiguous() const { return x.k_contiguous(); }
};
struct ViewSym {
  const float *p;
  long ld;
  bool upper;
  __device__ float operator()(int r, int k) const {
    const bool stored = upper ? (k >= r) : (k <= r);
    return stored ? p[long(r) * ld + k] : p[long(k) * ld + r];
  }
  __device__ bool k_contiguous() const { return true; }
};

// Grouped split: job j slices one operand of one product (ViewPlain) into
// its three planes; the grid's blocks are the jobs' 32 x 32 tiles in job
// order, first[j] the first block of job j.
struct SplitJob {
  ViewPlain x;
  int rows, K, Rp, Kp;
  __nv_bfloat16 *out;
  long first;
};
__global__ void split3_group_kernel(const SplitJob *__restrict__ jobs, int njobs) {
  const long b = blockIdx.x;
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].first <= b) lo = mid;
    else hi = mid - 1;
  }
  const SplitJob &J = jobs[lo];
  const long local = b - J.first;
  const int kt = (J.Kp + 31) / 32;
  split3_tile(J.x, J.rows, J.K, J.Rp, J.Kp, J.out, int(local / kt) * 32, int(local % kt) * 32);
}

// ---------------------------------------------------------------- host ----
template <class Op>
static void split(Op X, int rows, int K, int Rp, int Kp, __nv_bfloat16 *out) {
  dim3 grid(unsigned(ceil_div(Kp, 32)), unsigned(ceil_div(Rp, 32)));
  split3_kernel<Op><<<grid, 256, 0, ctx().stream>>>(X, rows, K, Rp, Kp, out);
  EXB_LAUNCH("bf16 split kernel");
  count_launch();
}

static int round_up(long v, int m) { return int((v + m - 1) / m * m); }

// C (M x N) = alpha * X_A X_B^T + beta * C where X_A is M x K and X_B is
// N x K (both logical, row r / column k).  tri: syrk triangle; same_ab:
// X_B is X_A (syrk), split once.
template <class OA, class OB>
static void run(OA xa, OB xb, int M, int N, int K, float alpha, float beta, float *C, long ldc, int tri, bool same_ab) {
  Context &c = ctx();
  const int Kp = round_up(K, BK), Mp = round_up(M, BM), Np = round_up(N, BN);
  const size_t a_elems = size_t(kSlices) * Mp * Kp, b_elems = same_ab ? 0 : size_t(kSlices) * Np * Kp;
  char *ws = static_cast<char *>(scratch((a_elems + b_elems) * 2 + 256));
  __nv_bfloat16 *sa = reinterpret_cast<__nv_bfloat16 *>(ws);
  __nv_bfloat16 *sb = same_ab ? sa : sa + a_elems;
  split(xa, M, K, Mp, Kp, sa);
  if (!same_ab) split(xb, N, K, Np, Kp, sb);
  const CUtensorMap ma = make_map(sa, long(kSlices) * Mp, Kp, BK, BM);
  const CUtensorMap mb = make_map(sb, long(kSlices) * (same_ab ? Mp : Np), Kp, BK, BN);
  Params p;
  p.M = M;
  p.N = N;
  p.K = K;
  p.Mp = Mp;
  p.Np = same_ab ? Mp : Np;
  p.kblocks = Kp / BK;
  p.mtiles = Mp / BM;
  p.ntiles = Np / BN;
  p.tri = tri;
  p.tiles = tri ? p.mtiles * (p.mtiles + 1) / 2 : p.mtiles * p.ntiles;
  p.alpha = alpha;
  p.beta = beta;
  p.C = C;
  p.ldc = ldc;
  p.status = device_status_word();
  static std::once_flag attr[64];
  const int smem = kDynSmem;
  const int dev = c.device < 64 ? c.device : 63;
  std::call_once(attr[dev], [smem] {
    EXB_CUDA(cudaFuncSetAttribute(split_bf16_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  });
  const int grid = p.tiles < c.sm_count ? p.tiles : c.sm_count;
  split_bf16_gemm_kernel<<<grid, kThreads, smem, c.stream>>>(ma, mb, p);
  EXB_LAUNCH("split-bf16 tcgen05 gemm kernel");
  count_launch();
  c.status_pending = true;
}

// A group of sgemm products on the tensor cores: slice planes, split jobs,
// per-product tensor maps and the tile items, built once and kept on the
// device; a launch runs the grouped split and the grouped product.
constexpr int kGroupSmem = kDynSmem;

struct TcGroupState {
  TcGroupGemm *gg = nullptr;
  TcItem *items = nullptr;
  SplitJob *jobs = nullptr;
  __nv_bfloat16 *planes = nullptr;
  int nitems = 0, njobs = 0;
  long split_blocks = 0;
};

static TcGroupState *group_create(const TcGroupOp *ops, int n) {
  // launch set-up done here, outside any stream capture of the launches
  {
    static std::once_flag attr[64];
    const int dev = ctx().device < 64 ? ctx().device : 63;
    std::call_once(attr[dev], [] {
      EXB_CUDA(cudaFuncSetAttribute(split_bf16_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kGroupSmem));
    });
    (void)device_status_word();
  }
  std::vector<TcGroupGemm> gg(n);
  std::vector<SplitJob> jobs;
  std::vector<std::pair<int, TcItem>> items;  // (k-blocks, item)
  std::vector<size_t> aoff(n), boff(n);
  size_t total = 0;
  for (int g = 0; g < n; ++g) {
    const TcGroupOp &o = ops[g];
    const int Kp = round_up(o.k, BK), Mp = round_up(o.m, BM), Np = round_up(o.n, BN);
    aoff[g] = total;
    total += size_t(kSlices) * Mp * Kp;
    boff[g] = total;
    total += size_t(kSlices) * Np * Kp;
  }
  TcGroupState *st = new TcGroupState();
  cudaError_t e = cudaMalloc(&st->planes, (total ? total : 1) * 2);
  if (e != cudaSuccess) {
    cudaGetLastError();
    delete st;
    fail(EXOBLAS_ALLOC_FAILED, "tensor-core batch: slice planes");
  }
  long first = 0;
  for (int g = 0; g < n; ++g) {
    const TcGroupOp &o = ops[g];
    const int Kp = round_up(o.k, BK), Mp = round_up(o.m, BM), Np = round_up(o.n, BN);
    __nv_bfloat16 *pa = st->planes + aoff[g], *pb = st->planes + boff[g];
    // op(B) is k x n; its K-major form is row j, column kk = op(B)[kk][j]
    const SplitJob ja{ViewPlain{o.A, o.lda, o.ta}, o.m, o.k, Mp, Kp, pa, first};
    first += long(Mp / 32) * ((Kp + 31) / 32);
    const SplitJob jb{ViewPlain{o.B, o.ldb, !o.tb}, o.n, o.k, Np, Kp, pb, first};
    first += long(Np / 32) * ((Kp + 31) / 32);
    jobs.push_back(ja);
    jobs.push_back(jb);
    TcGroupGemm &q = gg[g];
    q.ma = make_map(pa, long(kSlices) * Mp, Kp, BK, BM);
    q.mb = make_map(pb, long(kSlices) * Np, Kp, BK, BN);
    q.M = o.m;
    q.N = o.n;
    q.Mp = Mp;
    q.Np = Np;
    q.kblocks = Kp / BK;
    q.alpha = o.alpha;
    q.beta = o.beta;
    q.C = o.C;
    q.ldc = o.ldc;
    for (int mt = 0; mt < Mp / BM; ++mt)
      for (int nt = 0; nt < Np / BN; ++nt) items.push_back({q.kblocks, TcItem{g, mt, nt, 0}});
  }
  // longest tiles first; ties keep product and raster order (stable)
  std::stable_sort(items.begin(), items.end(),
                   [](const std::pair<int, TcItem> &a, const std::pair<int, TcItem> &b) { return a.first > b.first; });
  if (first > 0x7fffffffL) {
    cudaFree(st->planes);
    delete st;
    fail(EXOBLAS_INVALID_VALUE, "tensor-core batch: too many split tiles for one launch");
  }
  std::vector<TcItem> it(items.size());
  for (size_t i = 0; i < items.size(); ++i) it[i] = items[i].second;
  st->nitems = int(it.size());
  st->njobs = int(jobs.size());
  st->split_blocks = first;
  e = cudaMalloc(&st->gg, sizeof(TcGroupGemm) * (n ? n : 1));
  if (e == cudaSuccess) e = cudaMalloc(&st->items, sizeof(TcItem) * (it.empty() ? 1 : it.size()));
  if (e == cudaSuccess) e = cudaMalloc(&st->jobs, sizeof(SplitJob) * (jobs.empty() ? 1 : jobs.size()));
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaFree(st->planes);
    cudaFree(st->gg);
    cudaFree(st->items);
    cudaFree(st->jobs);
    delete st;
    fail(EXOBLAS_ALLOC_FAILED, "tensor-core batch: tables");
  }
  Context &c = ctx();
  if (n) EXB_CUDA(cudaMemcpyAsync(st->gg, gg.data(), sizeof(TcGroupGemm) * n, cudaMemcpyHostToDevice, c.stream));
  if (!it.empty())
    EXB_CUDA(cudaMemcpyAsync(st->items, it.data(), sizeof(TcItem) * it.size(), cudaMemcpyHostToDevice, c.stream));
  if (!jobs.empty())
    EXB_CUDA(cudaMemcpyAsync(st->jobs, jobs.data(), sizeof(SplitJob) * jobs.size(), cudaMemcpyHostToDevice, c.stream));
  EXB_CUDA(cudaStreamSynchronize(c.stream));
  return st;
}

static int group_launch(const TcGroupState *st, cudaStream_t s) {
  if (!st || st->nitems == 0) return 0;
  Context &c = ctx();
  split3_group_kernel<<<unsigned(st->split_blocks), 256, 0, s>>>(st->jobs, st->njobs);
  EXB_LAUNCH("grouped bf16 split kernel");
  const int smem = kGroupSmem;
  const int grid = st->nitems < c.sm_count ? st->nitems : c.sm_count;
  split_bf16_group_kernel<<<grid, kThreads, smem, s>>>(st->gg, st->items, st->nitems, device_status_word());
  EXB_LAUNCH("grouped split-bf16 tcgen05 gemm kernel");
  c.status_pending = true;
  return 2;
}

static void group_destroy(TcGroupState *st) {
  if (!st) return;
  cudaFree(st->planes);
  cudaFree(st->gg);
  cudaFree(st->items);
  cudaFree(st->jobs);
  delete st;
}

}  // namespace t5

void gemm_split_bf16(bool ta, bool tb, long m, long n, long k, float alpha, const float *A, long lda, const float *B,
                     long ldb, float beta, float *C, long ldc) {
  if (m <= 0 || n <= 0) return;
  // op(B) is k x n; its K-major form is row j, column kk = op(B)[kk][j]
  t5::run(t5::ViewPlain{A, lda, ta}, t5::ViewPlain{B, ldb, !tb}, int(m), int(n), int(k), alpha, beta, C, ldc, 0,
          false);
}

void symm_split_bf16(bool left, bool upper, long m, long n, float alpha, const float *A, long lda, const float *B,
                     long ldb, float beta, float *C, long ldc) {
  if (m <= 0 || n <= 0) return;
  if (left)  // C = sym(A) B: X_A = sym(A) (m x m), X_B(j, kk) = B[kk][j]
    t5::run(t5::ViewSym{A, lda, upper}, t5::ViewPlain{B, ldb, true}, int(m), int(n), int(m), alpha, beta, C, ldc, 0,
            false);
  else  // C = B sym(A): X_A = B (m x n), X_B = sym(A) (n x n, symmetric)
    t5::run(t5::ViewPlain{B, ldb, false}, t5::ViewSym{A, lda, upper}, int(m), int(n), int(n), alpha, beta, C, ldc, 0,
            false);
}

void syrk_split_bf16(bool upper, bool trans, long n, long k, float alpha, const float *A, long lda, float beta,
                     float *C, long ldc) {
  if (n <= 0) return;
  // X_A = op(A) (n x k): NoTrans row i of A, Trans column i of A
  t5::ViewPlain x{A, lda, trans};
  t5::run(x, x, int(n), int(n), int(k), alpha, beta, C, ldc, upper ? 2 : 1, true);
}

void syr2k_split_bf16(bool upper, bool trans, long n, long k, float alpha, const float *A, long lda, const float *B,
                      long ldb, float beta, float *C, long ldc) {
  if (n <= 0) return;
  // X_A = [op(A) | op(B)], X_B = [op(B) | op(A)] (n x 2k each)
  const t5::ViewPlain a{A, lda, trans}, b{B, ldb, trans};
  t5::run(t5::ViewCat{a, b, int(k)}, t5::ViewCat{b, a, int(k)}, int(n), int(n), int(2 * k), alpha, beta, C, ldc,
          upper ? 2 : 1, false);
}

TcGroup *tc_group_create(const TcGroupOp *ops, int n) {
  return reinterpret_cast<TcGroup *>(t5::group_create(ops, n));
}
int tc_group_launch(const TcGroup *g, cudaStream_t s) {
  const int k = t5::group_launch(reinterpret_cast<const t5::TcGroupState *>(g), s);
  count_launch(k);
  return k;
}
void tc_group_destroy(TcGroup *g) { t5::group_destroy(reinterpret_cast<t5::TcGroupState *>(g)); }

}  // namespace l3
}  // namespace exb
