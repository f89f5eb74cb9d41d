// Batched execution of many independent, unevenly sized BLAS calls in one
// persistent launch: sgemm, dgemv and strsv (the reference's exo_sgemm,
// exo_dgemv and exo_strsv semantics, test/level3/gemm/exo_gemm_wrapper.h,
// test/level2/gemv/exo_gemv_wrapper.h, test/level2/trsv/exo_trsv_wrapper.h).
//
// sgemm calls of at least 128 in m, n and k run on the tensor cores instead:
// one grouped split-BF16 product over all of them (gemm_tc.cu), launched
// before the persistent kernel; each gives the bits of exo_sgemm on the
// split-BF16 path.  A plan turns the other calls into work units, each
// small enough for one CTA:
//   GEMM_TILE   one TM x TN tile of one sgemm, TM x TN chosen per call by the
//               autotuner (32x32, 64x64 or 128x128)
//   GEMV_ROWS   128 rows of a NoTrans dgemv / 64 columns of a Trans dgemv
//   TRSV        one whole strsv (blocked substitution inside the CTA)
// sorted longest-first (each unit's cost estimated from its flops and bytes)
// and uploaded once.  A run zeroes a ticket and launches the persistent
// kernel (grid = SMs x resident CTAs), whose CTAs claim units in order with
// atomicAdd.  Runs are capturable in a CUDA graph (exoblas_batch_graph).
// The autotuner measures each tile shape's saturated throughput per K
// bucket and picks, per call, the shape with the least estimated time
// (padding waste included); measurements are cached in a JSON file when
// EXOBLAS_TUNE_CACHE names one.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "batch.h"
#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace bt {

constexpr int kThreads = 256;

// Unit kinds.  The batch API's calls use the first four (sgemm tiles, dgemv
// rows / columns, strsv); the request server's device batches also use the
// other precision of each (dgemm / dsyrk tiles, sgemv, dtrsv).
enum UnitKind : int {
  kGemmTile = 0, kGemvRows = 1, kGemvCols = 2, kTrsv = 3,
  kDGemmTile = 4, kSGemvRows = 5, kSGemvCols = 6, kDTrsv = 7
};

struct Unit {
  int kind;
  int op;      // index into the op table
  int r0, c0;  // tile / strip origin
  int cfg;     // gemm tile config
};


// ------------------------------------------------------------ gemm tiles --
// One TM x TN tile of C = alpha op(A) op(B) + beta C: RM x RN outputs per
// thread, 16-deep K slices double-buffered in shared memory with the next
// slice prefetched into registers while the current one is multiplied.
template <typename T, int TM, int TN, int RM, int RN>
__device__ void gemm_tile(const Op &o, int m0, int n0, void *smv) {
  constexpr int BK = 16;
  constexpr int TX = TN / RN, TY = TM / RM;
  constexpr int LA = BK * TM / kThreads, LB = BK * TN / kThreads;
  static_assert(TX * TY == kThreads, "tile shape");
  T *sm = static_cast<T *>(smv);
  T *As = sm, *Bs = sm + 2 * BK * TM;  // [2][BK][TM], [2][BK][TN]
  const T *A = static_cast<const T *>(o.A), *B = static_cast<const T *>(o.B);
  T *C = static_cast<T *>(o.C);
  const bool ta = o.f0 != 111, tb = o.f1 != 111;
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  T ra[LA], rb[LB];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int s = 0; s < LA; ++s) {
      const int e = threadIdx.x + s * kThreads;
      const int kk = ta ? e / TM : e % BK, i = ta ? e % TM : e / BK;
      const long gi = m0 + i, gk = k0 + kk;
      ra[s] = (gi < o.m && gk < o.k) ? (ta ? A[gk * o.lda + gi] : A[gi * o.lda + gk]) : T(0);
    }
#pragma unroll
    for (int s = 0; s < LB; ++s) {
      const int e = threadIdx.x + s * kThreads;
      const int kk = tb ? e % BK : e / TN, j = tb ? e / BK : e % TN;
      const long gj = n0 + j, gk = k0 + kk;
      rb[s] = (gj < o.n && gk < o.k) ? (tb ? B[gj * o.ldb + gk] : B[gk * o.ldb + gj]) : T(0);
    }
  };
  auto stash = [&](int buf) {
#pragma unroll
    for (int s = 0; s < LA; ++s) {
      const int e = threadIdx.x + s * kThreads;
      const int kk = ta ? e / TM : e % BK, i = ta ? e % TM : e / BK;
      As[(buf * BK + kk) * TM + i] = ra[s];
    }
#pragma unroll
    for (int s = 0; s < LB; ++s) {
      const int e = threadIdx.x + s * kThreads;
      const int kk = tb ? e % BK : e / TN, j = tb ? e / BK : e % TN;
      Bs[(buf * BK + kk) * TN + j] = rb[s];
    }
  };
  T acc[RM][RN];
#pragma unroll
  for (int i = 0; i < RM; ++i)
#pragma unroll
    for (int j = 0; j < RN; ++j) acc[i][j] = T(0);
  __syncthreads();  // the previous unit may still read shared memory
  fetch(0);
  stash(0);
  __syncthreads();
  int buf = 0;
  for (int k0 = 0; k0 < o.k; k0 += BK) {
    const bool more = k0 + BK < o.k;
    if (more) fetch(k0 + BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[RM], b[RN];
#pragma unroll
      for (int i = 0; i < RM; ++i) a[i] = As[(buf * BK + kk) * TM + ty * RM + i];
#pragma unroll
      for (int j = 0; j < RN; ++j) b[j] = Bs[(buf * BK + kk) * TN + tx + j * TX];
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < RN; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    if (more) stash(buf ^ 1);
    buf ^= 1;
    __syncthreads();
  }
  const T alpha = T(o.alpha), beta = T(o.beta);
#pragma unroll
  for (int i = 0; i < RM; ++i) {
    const long gi = m0 + ty * RM + i;
    if (gi >= o.m) continue;
#pragma unroll
    for (int j = 0; j < RN; ++j) {
      const long gj = n0 + tx + j * TX;
      if (gj >= o.n) continue;
      if ((o.tri == 1 && gj > gi) || (o.tri == 2 && gj < gi)) continue;  // outside syrk's triangle
      T *c = C + gi * o.ldc + gj;
      *c = alpha * acc[i][j] + beta * *c;
    }
  }
}

// -------------------------------------------------------------- gemv -------
// NoTrans: rows [r0, r0+128) of y = beta y + alpha A x, a warp per row.
template <typename T>
__device__ void gemv_rows(const Op &o, int r0) {
  const T *A = static_cast<const T *>(o.A), *x = static_cast<const T *>(o.B);
  T *y = static_cast<T *>(o.C);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long incx = o.ldb, incy = o.ldc;
  const T *xb = incx < 0 ? x + (1 - long(o.n)) * incx : x;
  T *yb = incy < 0 ? y + (1 - long(o.m)) * incy : y;
  for (int r = r0 + warp; r < r0 + 128 && r < o.m; r += kThreads / 32) {
    const T *a = A + long(r) * o.lda;
    T s0 = 0, s1 = 0;
    int j = lane;
    for (; j + 32 < o.n; j += 64) {
      s0 = fma(a[j], xb[j * incx], s0);
      s1 = fma(a[j + 32], xb[(j + 32) * incx], s1);
    }
    if (j < o.n) s0 = fma(a[j], xb[j * incx], s0);
    T s = s0 + s1;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (lane == 0) {
      T *yr = yb + long(r) * incy;
      *yr = T(o.alpha) * s + T(o.beta) * *yr;
    }
  }
}
// Trans: columns [c0, c0+64) of y = beta y + alpha A^T x (A is m x n,
// y has n entries).  Lane quad q = tid / 4 owns column c0 + q; its four
// lanes take rows i = 4t + (tid % 4) and combine with two shuffles in a
// fixed order, so no shared memory or block barrier is involved.
template <typename T>
__device__ void gemv_cols(const Op &o, int c0) {
  const T *A = static_cast<const T *>(o.A), *x = static_cast<const T *>(o.B);
  T *y = static_cast<T *>(o.C);
  const long incx = o.ldb, incy = o.ldc;
  const T *xb = incx < 0 ? x + (1 - long(o.m)) * incx : x;
  T *yb = incy < 0 ? y + (1 - long(o.n)) * incy : y;
  const int col = threadIdx.x >> 2, grp = threadIdx.x & 3;
  const long j = c0 + col;
  T s = 0;
  if (j < o.n)
    for (int i = grp; i < o.m; i += 4) s = fma(A[long(i) * o.lda + j], xb[i * incx], s);
  s += __shfl_xor_sync(0xffffffffu, s, 1);
  s += __shfl_xor_sync(0xffffffffu, s, 2);
  if (grp == 0 && j < o.n) {
    T *yj = yb + j * incy;
    *yj = T(o.alpha) * s + T(o.beta) * *yj;
  }
}

// -------------------------------------------------------------- trsv -------
// One whole strsv in one CTA: 32-row blocks; the 8 warps update the next
// block's right-hand side with the solved prefix (row dots), then warp 0
// substitutes through the 32 x 32 diagonal block with shuffles.  Effective
// lower formulation as in trsv.cu.
template <typename T>
__device__ void trsv_cta(const Op &o, void *smv) {
  const T *A = static_cast<const T *>(o.A);
  T *x = static_cast<T *>(o.C);
  const long n = o.m, lda = o.lda, inc = o.ldc;
  T *xb = inc < 0 ? x + (1 - n) * inc : x;
  const bool upper = o.f0 == 121, trans = o.f1 != 111, unit = o.f2 != 131;
  const bool rev = upper != trans;
  auto cidx = [&](long k) { return rev ? n - 1 - k : k; };
  auto L = [&](long i, long j) -> T {
    const long ci = cidx(i), cj = cidx(j);
    return trans ? A[cj * lda + ci] : A[ci * lda + cj];
  };
  T *z = static_cast<T *>(smv);  // solved values in effective order (n <= 4096)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long b0 = 0; b0 < n; b0 += 32) {
    const long rows = n - b0 < 32 ? n - b0 : 32;
    // rhs for the block: b - L[b0.., 0:b0] z[0:b0], four rows per warp
    for (int r = warp; r < rows; r += kThreads / 32) {
      const long i = b0 + r;
      T s = T(0);
      for (long j = lane; j < b0; j += 32) s = fma(L(i, j), z[j], s);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
      if (lane == 0) z[i] = xb[cidx(i) * inc] - s;
    }
    __syncthreads();
    if (warp == 0) {
      T v = lane < rows ? z[b0 + lane] : T(0);
      for (int j = 0; j < rows; ++j) {
        T xj = v;
        if (lane == j && !unit) xj = v / L(b0 + j, b0 + j);
        xj = __shfl_sync(0xffffffffu, xj, j);
        if (lane == j) v = xj;
        if (lane > j && lane < rows) v = fma(-L(b0 + lane, b0 + j), xj, v);
      }
      if (lane < rows) z[b0 + lane] = v;
    }
    __syncthreads();
  }
  for (long i = threadIdx.x; i < n; i += kThreads) xb[cidx(i) * inc] = z[i];
}

// ---------------------------------------------------------------- kernel --
__global__ void __launch_bounds__(kThreads)
    batch_kernel(const Op *__restrict__ ops, const Unit *__restrict__ units, int nunits, int *ticket) {
  extern __shared__ __align__(16) float smem_f[];
  __shared__ int s_u;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_u = atomicAdd(ticket, 1);
    __syncthreads();
    const int u = s_u;
    if (u >= nunits) return;
    const Unit un = units[u];
    const Op o = ops[un.op];
    switch (un.kind) {
      case kGemmTile:
        if (un.cfg == 0)
          gemm_tile<float, 32, 32, 2, 2>(o, un.r0, un.c0, smem_f);
        else if (un.cfg == 1)
          gemm_tile<float, 64, 64, 4, 4>(o, un.r0, un.c0, smem_f);
        else
          gemm_tile<float, 128, 128, 8, 8>(o, un.r0, un.c0, smem_f);
        break;
      case kDGemmTile:  // 64 x 64: the FP64 operand slices fill the same shared memory
        gemm_tile<double, 64, 64, 4, 4>(o, un.r0, un.c0, smem_f);
        break;
      case kGemvRows:
        gemv_rows<double>(o, un.r0);
        break;
      case kGemvCols:
        gemv_cols<double>(o, un.c0);
        break;
      case kSGemvRows:
        gemv_rows<float>(o, un.r0);
        break;
      case kSGemvCols:
        gemv_cols<float>(o, un.c0);
        break;
      case kDTrsv:
        trsv_cta<double>(o, smem_f);
        break;
      default:
        trsv_cta<float>(o, smem_f);
        break;
    }
  }
}

constexpr size_t kSmem = 2 * 16 * (128 + 128) * 4 > 4096 * 4 ? 2 * 16 * (128 + 128) * 4 : 4096 * 4;

// --------------------------------------------------------------- tuner -----
// The autotuner measures, for every tile shape and K bucket (K = 16 * 2^b),
// the saturated throughput of that tile shape: one launch of enough tiles to
// fill every SM (a 2048 x 2048 output), timed with CUDA events after a
// warm-up.  A call (m, n, k) then gets the shape minimising
//   ceil(m / TM) ceil(n / TN) TM TN k / throughput(shape, bucket(k)),
// i.e. measured speed with the padding waste of the shape counted in.
const int kTiles[3][2] = {{32, 32}, {64, 64}, {128, 128}};

static int bucket(int v) {
  int b = 0;
  while (b < 7 && (16 << (b + 1)) <= v) ++b;
  return b;  // 16..31 -> 0, ..., >= 2048 -> 7
}

struct Tuner {
  std::mutex mu;
  bool loaded = false;
  bool tuned = false;
  double gflops[3][8];  // measured throughput per [tile shape][K bucket]
  Tuner() {
    // untuned defaults (GFLOP/s): larger tiles reuse more per byte
    for (int b = 0; b < 8; ++b) {
      gflops[0][b] = 6000;
      gflops[1][b] = 14000;
      gflops[2][b] = 22000;
    }
  }
};
static Tuner g_tuner;

static const char *cache_path() {
  const char *p = getenv("EXOBLAS_TUNE_CACHE");
  return p && *p ? p : nullptr;
}

// cache format: {"batch_sgemm_gflops": [[t00, ..., t07], [t10, ...], [t20, ...]]}
static void load_cache() {
  if (g_tuner.loaded) return;
  g_tuner.loaded = true;
  const char *path = cache_path();
  if (!path) return;
  FILE *f = fopen(path, "r");
  if (!f) return;
  char buf[4096];
  const size_t nr = fread(buf, 1, sizeof buf - 1, f);
  fclose(f);
  buf[nr] = 0;
  const char *p = strstr(buf, "batch_sgemm_gflops");
  if (!p) return;
  double v[3][8];
  for (int i = 0; i < 3; ++i) {
    p = strchr(p + 1, '[');
    if (!p) return;
    if (i == 0) {
      p = strchr(p + 1, '[');
      if (!p) return;
    }
    ++p;
    for (int j = 0; j < 8; ++j) {
      char *end = nullptr;
      v[i][j] = strtod(p, &end);
      if (end == p || !(v[i][j] > 0)) return;
      p = end;
      while (*p == ',' || *p == ' ') ++p;
    }
  }
  memcpy(g_tuner.gflops, v, sizeof v);
  g_tuner.tuned = true;
}

static void save_cache() {
  const char *path = cache_path();
  if (!path) return;
  FILE *f = fopen(path, "w");
  if (!f) return;
  fprintf(f, "{\"batch_sgemm_gflops\": [");
  for (int i = 0; i < 3; ++i) {
    fprintf(f, "%s[", i ? ", " : "");
    for (int j = 0; j < 8; ++j) fprintf(f, "%s%.1f", j ? ", " : "", g_tuner.gflops[i][j]);
    fprintf(f, "]");
  }
  fprintf(f, "]}\n");
  fclose(f);
}

static int launch_units(const Op *dops, const Unit *dunits, int nunits, int *ticket, cudaStream_t s, int sms);

static void tune_all() {
  Context &c = ctx();
  const int d = 2048, kmax = 2048;
  float *a = nullptr, *b = nullptr, *cm = nullptr;
  Op *dop = nullptr;
  Unit *du = nullptr;
  int *tk = nullptr;
  const int maxunits = (d / 32) * (d / 32);
  EXB_CUDA(cudaMalloc(&a, size_t(d) * kmax * 4));
  EXB_CUDA(cudaMalloc(&b, size_t(d) * kmax * 4));
  EXB_CUDA(cudaMalloc(&cm, size_t(d) * d * 4));
  EXB_CUDA(cudaMalloc(&dop, sizeof(Op)));
  EXB_CUDA(cudaMalloc(&du, sizeof(Unit) * maxunits));
  EXB_CUDA(cudaMalloc(&tk, 4));
  EXB_CUDA(cudaMemsetAsync(a, 0, size_t(d) * kmax * 4, c.stream));
  EXB_CUDA(cudaMemsetAsync(b, 0, size_t(d) * kmax * 4, c.stream));
  cudaEvent_t e0, e1;
  EXB_CUDA(cudaEventCreate(&e0));
  EXB_CUDA(cudaEventCreate(&e1));
  std::vector<Unit> us;
  for (int cf = 0; cf < 3; ++cf) {
    const int TM = kTiles[cf][0], TN = kTiles[cf][1];
    us.clear();
    for (int i = 0; i < d; i += TM)
      for (int j = 0; j < d; j += TN) us.push_back(Unit{kGemmTile, 0, i, j, cf});
    EXB_CUDA(cudaMemcpyAsync(du, us.data(), sizeof(Unit) * us.size(), cudaMemcpyHostToDevice, c.stream));
    for (int bk = 0; bk < 8; ++bk) {
      const int kk = 16 << bk;
      Op o{};
      o.op = 1;
      o.f0 = o.f1 = 111;
      o.m = o.n = d;
      o.k = kk;
      o.alpha = 1;
      o.beta = 0;
      o.A = a;
      o.lda = kk;
      o.B = b;
      o.ldb = d;
      o.C = cm;
      o.ldc = d;
      EXB_CUDA(cudaMemcpyAsync(dop, &o, sizeof o, cudaMemcpyHostToDevice, c.stream));
      launch_units(dop, du, int(us.size()), tk, c.stream, c.sm_count);  // warm-up
      EXB_CUDA(cudaEventRecord(e0, c.stream));
      launch_units(dop, du, int(us.size()), tk, c.stream, c.sm_count);
      EXB_CUDA(cudaEventRecord(e1, c.stream));
      EXB_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      EXB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      g_tuner.gflops[cf][bk] = 2.0 * d * double(d) * kk / (double(ms) * 1e-3) / 1e9;
    }
  }
  g_tuner.tuned = true;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(a);
  cudaFree(b);
  cudaFree(cm);
  cudaFree(dop);
  cudaFree(du);
  cudaFree(tk);
  save_cache();
}

static int tile_config(int m, int n, int k) {
  std::lock_guard<std::mutex> lk(g_tuner.mu);
  load_cache();
  const int bk = bucket(k > 0 ? k : 1);
  int best = 0;
  double best_t = 1e300;
  for (int cf = 0; cf < 3; ++cf) {
    const double TM = kTiles[cf][0], TN = kTiles[cf][1];
    const double work = std::ceil(m / TM) * std::ceil(n / TN) * TM * TN * double(k > 0 ? k : 1) * 2.0;
    const double t = work / (g_tuner.gflops[cf][bk] * 1e9);
    if (t < best_t * 0.98) {  // prefer the larger tile on near-ties
      best_t = t;
      best = cf;
    } else if (t < best_t * 1.02) {
      best = cf;
      best_t = std::min(best_t, t);
    }
  }
  return best;
}

static int launch_units(const Op *dops, const Unit *dunits, int nunits, int *ticket, cudaStream_t s, int sms) {
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 64 && !attr[dev]) {
    EXB_CUDA(cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kSmem)));
    attr[dev] = true;
  }
  int per_sm = 0;
  EXB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, kThreads, kSmem));
  int grid = sms * (per_sm > 0 ? per_sm : 1);
  if (grid > nunits) grid = nunits;
  if (grid < 1) return 0;
  EXB_CUDA(cudaMemsetAsync(ticket, 0, 4, s));
  batch_kernel<<<grid, kThreads, kSmem, s>>>(dops, dunits, nunits, ticket);
  EXB_LAUNCH("batch kernel");
  count_launch();
  return grid;
}

// ------------------------------------------------------------------ plan ---
// sgemm calls of at least kTcMN in m and n and kTcK in k go to the tensor
// cores as one grouped split-BF16 product (l3::tc_group_*) unless switched
// off; the rest become work units of the persistent kernel.
static std::atomic<bool> g_tensor_cores{true};
constexpr int kTcMN = 128, kTcK = 128;
static bool tc_eligible(const exoblas_batch_op &b) {
  return g_tensor_cores && b.op == EXOBLAS_BATCH_SGEMM && b.m >= kTcMN && b.n >= kTcMN && b.k >= kTcK;
}

struct Plan {
  int device = 0;
  l3::TcGroup *tc = nullptr;  // sgemm calls on the tensor cores
  int ntc = 0;
  Op *ops = nullptr;
  Unit *units = nullptr;
  int *ticket = nullptr;
  int nunits = 0, nops = 0;
  double flops = 0, bytes = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t graph_stream = nullptr;
};

static double unit_cost(const exoblas_batch_op &b, int kind, int cfg) {
  // seconds-like score: flops at ~40 TF/s FP32, bytes at ~6 TB/s, trsv chain
  switch (kind) {
    case kGemmTile: {
      const double t = kTiles[cfg][0] * double(kTiles[cfg][1]);
      return 2.0 * t * b.k / 4e13 + 1e-6;
    }
    case kGemvRows:
      return 128.0 * b.n * 8 / 6e12 + 1e-6;
    case kGemvCols:
      return 64.0 * b.m * 8 / 6e12 + 1e-6;
    default:
      return double(b.m) * b.m / 2 / 5e10 + b.m * 5e-8;  // one CTA, FP32 chain
  }
}

// Work units of one call, appended to `us` with their estimated cost.
// Returns false for an op code it does not know.
static bool add_units(const Op &o, int idx, std::vector<std::pair<double, Unit>> &us, double &flops, double &bytes) {
  exoblas_batch_op b{};  // cost model view
  b.m = o.m;
  b.n = o.n;
  b.k = o.k;
  auto tiles = [&](int kind, int cfg, int TM, int TN) {
    for (int r = 0; r < o.m; r += TM)
      for (int cc = 0; cc < o.n; cc += TN) {
        if (o.tri == 1 && cc > r + TM - 1) continue;  // tile entirely above the lower triangle
        if (o.tri == 2 && cc + TN - 1 < r) continue;  // entirely below the upper triangle
        us.push_back({unit_cost(b, kGemmTile, cfg), Unit{kind, idx, r, cc, cfg}});
      }
  };
  switch (o.op) {
    case EXOBLAS_BATCH_SGEMM:
    case kOpSSyrk: {
      if (o.m == 0 || o.n == 0) break;
      const int cf = tile_config(o.m, o.n, o.k);
      tiles(kGemmTile, cf, kTiles[cf][0], kTiles[cf][1]);
      flops += 2.0 * o.m * o.n * o.k;
      break;
    }
    case kOpDGemm:
    case kOpDSyrk:
      if (o.m == 0 || o.n == 0) break;
      tiles(kDGemmTile, 1, 64, 64);
      flops += 2.0 * o.m * o.n * o.k;
      break;
    case EXOBLAS_BATCH_DGEMV:
    case kOpSGemv: {
      if (o.m == 0 || o.n == 0) break;
      const bool dbl = o.op == EXOBLAS_BATCH_DGEMV;
      if (o.f0 == 111) {
        for (int r = 0; r < o.m; r += 128)
          us.push_back({unit_cost(b, kGemvRows, 0), Unit{dbl ? kGemvRows : kSGemvRows, idx, r, 0, 0}});
      } else {
        for (int cc = 0; cc < o.n; cc += 64)
          us.push_back({unit_cost(b, kGemvCols, 0), Unit{dbl ? kGemvCols : kSGemvCols, idx, 0, cc, 0}});
      }
      bytes += (double(o.m) * o.n + o.m + 2.0 * o.n) * (dbl ? 8 : 4);
      break;
    }
    case EXOBLAS_BATCH_STRSV:
    case kOpDTrsv: {
      if (o.m == 0) break;
      const bool dbl = o.op == kOpDTrsv;
      us.push_back({unit_cost(b, kTrsv, 0) * (dbl ? 8 : 1), Unit{dbl ? kDTrsv : kTrsv, idx, 0, 0, 0}});
      bytes += (double(o.m) * (o.m + 1) / 2 + 2.0 * o.m) * (dbl ? 8 : 4);
      break;
    }
    default:
      return false;
  }
  return true;
}

// One device batch at a time on the runner's own stream: the request
// server's continuous batching of small requests.
struct TickRunner {
  int device = 0;
  cudaStream_t stream = nullptr;
  Op *dops = nullptr;
  Unit *dunits = nullptr;
  int *ticket = nullptr;
  size_t cap_ops = 0, cap_units = 0;
  void *pinned = nullptr;
  size_t cap_pinned = 0;
};

TickRunner *tick_create() {
  TickRunner *t = new TickRunner();
  EXB_CUDA(cudaGetDevice(&t->device));
  EXB_CUDA(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking));
  EXB_CUDA(cudaMalloc(&t->ticket, 256));
  return t;
}

void tick_destroy(TickRunner *t) {
  if (!t) return;
  cudaStreamSynchronize(t->stream);
  cudaFree(t->dops);
  cudaFree(t->dunits);
  cudaFree(t->ticket);
  cudaFreeHost(t->pinned);
  cudaStreamDestroy(t->stream);
  cudaGetLastError();
  delete t;
}

bool tick_run(TickRunner *t, const std::vector<Op> &ops, int sm_count) {
  std::vector<std::pair<double, Unit>> us;
  double flops = 0, bytes = 0;
  for (size_t i = 0; i < ops.size(); ++i)
    if (!add_units(ops[i], int(i), us, flops, bytes)) return false;
  if (us.empty()) return true;
  std::stable_sort(us.begin(), us.end(), [](const std::pair<double, Unit> &a, const std::pair<double, Unit> &b) {
    return a.first > b.first;
  });
  auto grow = [](void **p, size_t &cap, size_t need) {
    if (need <= cap) return;
    if (*p) cudaFree(*p);
    *p = nullptr;
    cap = need + need / 2;
    EXB_CUDA(cudaMalloc(p, cap));
  };
  const size_t ob = sizeof(Op) * ops.size(), ub = sizeof(Unit) * us.size();
  grow(reinterpret_cast<void **>(&t->dops), t->cap_ops, ob);
  grow(reinterpret_cast<void **>(&t->dunits), t->cap_units, ub);
  if (ob + ub > t->cap_pinned) {
    if (t->pinned) EXB_CUDA(cudaFreeHost(t->pinned));
    t->cap_pinned = (ob + ub) * 2;
    EXB_CUDA(cudaHostAlloc(&t->pinned, t->cap_pinned, cudaHostAllocDefault));
  }
  char *h = static_cast<char *>(t->pinned);
  memcpy(h, ops.data(), ob);
  Unit *hu = reinterpret_cast<Unit *>(h + ob);
  for (size_t i = 0; i < us.size(); ++i) hu[i] = us[i].second;
  EXB_CUDA(cudaMemcpyAsync(t->dops, h, ob, cudaMemcpyHostToDevice, t->stream));
  EXB_CUDA(cudaMemcpyAsync(t->dunits, hu, ub, cudaMemcpyHostToDevice, t->stream));
  launch_units(t->dops, t->dunits, int(us.size()), t->ticket, t->stream, sm_count);
  EXB_CUDA(cudaStreamSynchronize(t->stream));
  return true;
}

}  // namespace bt
}  // namespace exb

using namespace exb;

extern "C" {

int exoblas_batch_tune(void) {
  return guarded("exoblas_batch_tune", [&] {
    std::lock_guard<std::mutex> lk(bt::g_tuner.mu);
    bt::load_cache();
    bt::tune_all();
  });
}

int exoblas_batch_plan_create(const exoblas_batch_op *ops, int count, exoblas_batch_plan *out) {
  return guarded("exoblas_batch_plan_create", [&] {
    if (!out) fail(EXOBLAS_INVALID_VALUE, "plan pointer is NULL");
    *out = nullptr;
    if (count < 0 || (count > 0 && !ops)) fail(EXOBLAS_INVALID_VALUE, "bad op list");
    Context &c = ctx();
    std::vector<bt::Op> dops(count);
    std::vector<std::pair<double, bt::Unit>> us;
    std::vector<l3::TcGroupOp> tcops;
    double flops = 0, bytes = 0;
    for (int i = 0; i < count; ++i) {
      const exoblas_batch_op &b = ops[i];
      bt::Op &o = dops[i];
      o.op = b.op;
      o.f0 = b.flags[0];
      o.f1 = b.flags[1];
      o.f2 = b.flags[2];
      o.m = b.m;
      o.n = b.n;
      o.k = b.k;
      o.alpha = b.alpha;
      o.beta = b.beta;
      o.A = b.A;
      o.lda = b.lda;
      o.B = b.B;
      o.ldb = b.ldb;
      o.C = b.C;
      o.ldc = b.ldc;
      if (b.m < 0 || b.n < 0 || b.k < 0) fail(EXOBLAS_INVALID_VALUE, "negative size in a batch op");
      for (const void *p : {b.A, b.B, static_cast<const void *>(b.C)})
        if (p && !is_device_pointer(p)) fail(EXOBLAS_INVALID_VALUE, "batch operands must be device pointers");
      switch (b.op) {
        case EXOBLAS_BATCH_SGEMM:
          break;
        case EXOBLAS_BATCH_DGEMV:
          if (b.m != 0 && b.n != 0 && (b.ldb == 0 || b.ldc == 0))
            fail(EXOBLAS_INVALID_VALUE, "zero vector stride in a batch dgemv");
          break;
        case EXOBLAS_BATCH_STRSV:
          if (b.m > 4096) fail(EXOBLAS_INVALID_VALUE, "batch strsv supports N <= 4096");
          if (b.m != 0 && b.ldc == 0) fail(EXOBLAS_INVALID_VALUE, "zero stride in a batch strsv");
          break;
        default:
          fail(EXOBLAS_INVALID_VALUE, "unknown batch op");
      }
      if (bt::tc_eligible(b)) {
        tcops.push_back(l3::TcGroupOp{b.flags[0] != 111, b.flags[1] != 111, b.m, b.n, b.k, float(b.alpha),
                                      float(b.beta), static_cast<const float *>(b.A), long(b.lda),
                                      static_cast<const float *>(b.B), long(b.ldb), static_cast<float *>(b.C),
                                      long(b.ldc)});
        flops += 2.0 * b.m * b.n * b.k;
        bytes += 4.0 * (double(b.m) * b.k + double(b.k) * b.n + 2.0 * b.m * b.n);
        continue;
      }
      bt::add_units(o, i, us, flops, bytes);
    }
    // longest first; ties keep submission order (stable)
    std::stable_sort(us.begin(), us.end(),
                     [](const std::pair<double, bt::Unit> &a, const std::pair<double, bt::Unit> &b) {
                       return a.first > b.first;
                     });
    std::vector<bt::Unit> units(us.size());
    for (size_t i = 0; i < us.size(); ++i) units[i] = us[i].second;
    bt::Plan *p = new bt::Plan();
    p->device = c.device;
    p->nops = count;
    p->nunits = int(units.size());
    p->flops = flops;
    p->bytes = bytes;
    cudaError_t e = cudaMalloc(&p->ops, sizeof(bt::Op) * (count ? count : 1));
    if (e == cudaSuccess) e = cudaMalloc(&p->units, sizeof(bt::Unit) * (units.empty() ? 1 : units.size()));
    if (e == cudaSuccess) e = cudaMalloc(&p->ticket, 256);
    if (e != cudaSuccess) {
      cudaGetLastError();
      cudaFree(p->ops);
      cudaFree(p->units);
      cudaFree(p->ticket);
      delete p;
      fail(EXOBLAS_ALLOC_FAILED, "batch plan allocation failed");
    }
    EXB_CUDA(cudaMemcpyAsync(p->ops, dops.data(), sizeof(bt::Op) * count, cudaMemcpyHostToDevice, c.stream));
    if (!units.empty())
      EXB_CUDA(cudaMemcpyAsync(p->units, units.data(), sizeof(bt::Unit) * units.size(), cudaMemcpyHostToDevice,
                               c.stream));
    EXB_CUDA(cudaStreamSynchronize(c.stream));
    if (!tcops.empty()) {
      try {
        p->tc = l3::tc_group_create(tcops.data(), int(tcops.size()));
      } catch (...) {
        cudaFree(p->ops);
        cudaFree(p->units);
        cudaFree(p->ticket);
        delete p;
        throw;
      }
      p->ntc = int(tcops.size());
    }
    *out = reinterpret_cast<exoblas_batch_plan>(p);
  });
}

int exoblas_batch_plan_run(exoblas_batch_plan plan) {
  return guarded("exoblas_batch_plan_run", [&] {
    bt::Plan *p = reinterpret_cast<bt::Plan *>(plan);
    if (!p) fail(EXOBLAS_INVALID_VALUE, "NULL plan");
    Context &c = ctx();
    if (c.device != p->device) fail(EXOBLAS_INVALID_VALUE, "plan belongs to another device");
    if (p->tc) l3::tc_group_launch(p->tc, c.stream);
    bt::launch_units(p->ops, p->units, p->nunits, p->ticket, c.stream, c.sm_count);
    if (c.blocking) EXB_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int exoblas_batch_plan_graph_launch(exoblas_batch_plan plan) {
  return guarded("exoblas_batch_plan_graph_launch", [&] {
    bt::Plan *p = reinterpret_cast<bt::Plan *>(plan);
    if (!p) fail(EXOBLAS_INVALID_VALUE, "NULL plan");
    Context &c = ctx();
    if (!p->exec) {
      // capture one run (tensor-core group, ticket reset + persistent
      // kernel) on a private stream; the status word the group's kernel
      // reports to is allocated first (no allocation while capturing)
      (void)device_status_word();
      EXB_CUDA(cudaStreamCreateWithFlags(&p->graph_stream, cudaStreamNonBlocking));
      EXB_CUDA(cudaStreamBeginCapture(p->graph_stream, cudaStreamCaptureModeThreadLocal));
      if (p->tc) l3::tc_group_launch(p->tc, p->graph_stream);
      bt::launch_units(p->ops, p->units, p->nunits, p->ticket, p->graph_stream, c.sm_count);
      EXB_CUDA(cudaStreamEndCapture(p->graph_stream, &p->graph));
      EXB_CUDA(cudaGraphInstantiate(&p->exec, p->graph, 0));
    }
    EXB_CUDA(cudaGraphLaunch(p->exec, c.stream));
    if (c.blocking) EXB_CUDA(cudaStreamSynchronize(c.stream));
  });
}

int exoblas_batch_plan_info(exoblas_batch_plan plan, int *units, double *flops, double *bytes) {
  return guarded("exoblas_batch_plan_info", [&] {
    bt::Plan *p = reinterpret_cast<bt::Plan *>(plan);
    if (!p) fail(EXOBLAS_INVALID_VALUE, "NULL plan");
    if (units) *units = p->nunits;
    if (flops) *flops = p->flops;
    if (bytes) *bytes = p->bytes;
  });
}

int exoblas_batch_plan_destroy(exoblas_batch_plan plan) {
  return guarded("exoblas_batch_plan_destroy", [&] {
    bt::Plan *p = reinterpret_cast<bt::Plan *>(plan);
    if (!p) return;
    cudaStreamSynchronize(ctx().stream);
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->graph_stream) cudaStreamDestroy(p->graph_stream);
    l3::tc_group_destroy(p->tc);
    cudaFree(p->ops);
    cudaFree(p->units);
    cudaFree(p->ticket);
    delete p;
  });
}

int exoblas_batch_set_tensor_cores(int on) {
  return guarded("exoblas_batch_set_tensor_cores", [&] { bt::g_tensor_cores = on != 0; });
}

int exoblas_batch_plan_tensor_core_calls(exoblas_batch_plan plan, int *calls) {
  return guarded("exoblas_batch_plan_tensor_core_calls", [&] {
    bt::Plan *p = reinterpret_cast<bt::Plan *>(plan);
    if (!p || !calls) fail(EXOBLAS_INVALID_VALUE, "NULL argument");
    *calls = p->ntc;
  });
}

int exoblas_batch_tile_config(int m, int n, int k) {
  int c = -1;
  guarded("exoblas_batch_tile_config", [&] { c = bt::tile_config(m, n, k); });
  return c;
}

}  // extern "C"
