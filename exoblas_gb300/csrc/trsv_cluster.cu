// Triangular solve (src/level2/trsv.py:10-52) for large n: blocked
// substitution in one persistent launch of 16-CTA thread-block clusters
// (8-CTA where fewer than four 16-CTA clusters fit).
//
// Effective-lower formulation as in trsv.cu: L(i, j) = trans ? A[c(j)][c(i)]
// : A[c(i)][c(j)], c(k) = rev ? n-1-k : k, z = x in effective order.  Blocks
// of kTB = 64 rows.  Roles, decided at run time so that the solver is always
// a cluster that is already running:
//
//  * the first cluster to start is the SOLVER.  Each of its C CTAs owns
//    64/C rows of every block.  Step K: rhs = b_K - (bulk partial sums of
//    block row K) - L[K,K-kD..K-1] x, exchanged between the C CTAs through
//    distributed shared memory, then x_K = inv(L_KK) rhs
//    (the diagonal block solved in shared memory with its inverse, computed
//    beforehand by trsv_inverse_kernel in the working precision), exchanged
//    again and published to global memory with a release flag.  With
//    8-CTA clusters (solve_chain) everything except the L[K,K-1] product
//    and the two exchanges runs in the shadow of the previous step's cluster
//    barrier; with 16-CTA clusters (solve_chain2) dedicated critical and
//    helper warps exchange through st.async stores counted on mbarriers.
//    The operand rows the solver needs are prefetched with cp.async.
//    A 16-CTA solver CTA also has a publisher warp (x_m to global memory
//    with its release flag) and two slot-loader warps (even and odd block
//    rows: sum the streamers' slots of each block row ahead of time into
//    shared memory), so no global-memory round trip sits on the helpers'
//    loop.
//  * every other CTA STREAMS the bulk, tiles L[K, J] with J < K - kD.  Row
//    K's bulk is split into full chunks of kCT tiles and a tail holding its
//    newest tiles; each work item writes its 64 partial row sums to its
//    slot (K, c) and sets the slot's flag, and the solver adds the slots of
//    block row K in slot order, so results are deterministic.  Tail workers
//    (the first kTailCTAs of each streaming cluster) take tails in order of
//    K, chunk workers take full chunks in order of readiness.  Extra
//    streaming CTAs on a side stream use the SMs that the clusters leave
//    free.
// Deadlock freedom: the solver only waits on items, which are claimed in
// order by running CTAs and themselves only wait on the solver's x flags;
// streamers only wait on the solver, which is running.  Every wait is
// bounded: on expiry the CTA records the timeout in the device status word,
// stops waiting for the rest of the launch, and the host reports
// EXOBLAS_TIMEOUT.  Solver CTAs keep arriving at every cluster barrier so the
// cluster always completes.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace cg = cooperative_groups;

namespace exb {
namespace l2 {

namespace tc {

constexpr int kTB = 64;            // block size
constexpr int kNT = 256;           // threads of a streaming CTA and of the 8-CTA solver
constexpr int kNTS = 352;          // threads per CTA of a 16-CTA launch: 8 solver warps, publisher, 2 slot loaders
constexpr int kCT = 4;             // tiles per streamer chunk
static_assert(kCT <= 32, "one ballot bit per tile of an item");
constexpr int kTailCTAs = 2;       // tail workers per streaming cluster
constexpr int kD = 6;              // near tiles done by the solver: J = K-1 .. K-kD
constexpr int kPre = 4;            // solver prefetch depth (steps)
constexpr int kXR = 8;             // x ring depth (>= kD + 1)
constexpr long long kSpin = 1ll << 24;

template <typename T>
struct alignas(16) SmemStream {
  // row pitch 64 + 64 / sizeof(T) elements: 16-byte row starts, and a row
  // step of 4 mod 8 sixteen-byte bank groups (see stream_items)
  static constexpr int kTP = kTB + 64 / int(sizeof(T));
  T tile[3][kTB][kTP];  // three stages: tiles load two ahead of the one in use
  alignas(16) T zs[kCT][kTB];  // x blocks of an item
};

template <typename T>
struct Args {
  long n;
  const T *A;
  long lda;
  T *z;
  const T *inv;  // nb x kTB x kTB
  T *slots;      // nb x nch x kTB
  int *xflag;    // nb
  int *sflag;    // nb x nch
  int *ctl;      // [0] solver claim, [1] chunk ticket, [2] tail ticket, [3] resident clusters
  int *status;
  int nb, nch;
  int nclusters;  // clusters of the clustered launch
  bool rev, trans, unit;
  bool vec16;  // rows of L are contiguous, 16-byte aligned runs of A (lower no-trans, even lda)
};

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

template <typename T>
__device__ __forceinline__ void cp_async(T *smem, const T *gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if constexpr (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// global index of effective element L(i, j) (both < n); A row-major
template <typename T>
__device__ __forceinline__ long lidx(const Args<T> &a, long i, long j) {
  const long ci = a.rev ? a.n - 1 - i : i, cj = a.rev ? a.n - 1 - j : j;
  return a.trans ? cj * a.lda + ci : ci * a.lda + cj;
}
template <typename T>
__device__ __forceinline__ long zidx(const Args<T> &a, long i) {
  return a.rev ? a.n - 1 - i : i;
}

// Bounded wait for *p != 0 by thread 0; returns false (and records the
// timeout) when it expires.
__device__ __forceinline__ bool wait_flag(const int *p, int *status, bool &dead) {
  if (dead) return false;
  long long spins = 0;
  while (ld_acquire(p) == 0) {
    if (++spins > kSpin) {
      atomicExch(status, 1);
      dead = true;
      return false;
    }
    __nanosleep(64);
  }
  return true;
}

// Bulk of block row K (kD < K): tiles J < K - kD.  It splits into full
// chunks c = 0 .. nfull(K)-1 of kCT tiles (J = kCT*c .. kCT*c + kCT-1) and a
// tail of 1 .. kCT tiles ending at the newest tile J = K-kD-1.  The solver
// adds the row's slots in order: its full chunks, then its tail.
__device__ __host__ __forceinline__ int nfull(long K) { return K > kD ? int((K - kD - 1) / kCT) : 0; }
__device__ __host__ __forceinline__ int nslots_row(long K) { return K > kD ? nfull(K) + 1 : 0; }
// full chunks in groups c' < c, group c' holding chunk c' of every row that
// has it (rows K >= kCT*(c'+1) + kD + 1), in increasing K
__device__ __host__ __forceinline__ long chunks_in_groups_before(long c, long nb) {
  const long M = nb - kCT - kD - 1;  // rows of group 0
  if (M <= 0) return 0;
  const long imax = (M + kCT - 1) / kCT;
  const long cc = c < imax ? c : imax;
  return cc * M - kCT * cc * (cc - 1) / 2;
}
__device__ __host__ __forceinline__ long chunk_items(long nb) { return chunks_in_groups_before(nb, nb); }
__device__ __host__ __forceinline__ long tail_items(long nb) { return nb - 1 - kD > 0 ? nb - 1 - kD : 0; }

// ------------------------------------------------------------ streamers ----
// Two kinds of streaming CTA.  Tail workers (the first kTailCTAs of every
// streaming cluster) take the rows' tails in order of K: the tail of row K
// holds the newest tiles, needed kD steps after x_{K-kD-1} appears, and a
// tail worker computes each tile as soon as its x block is published.
// Chunk workers take full chunks in order of the step that makes them ready
// (chunk c is ready once x_{kCT*c + kCT-1} is published; within a group, rows
// in increasing K).  A full chunk is never among a row's newest tiles, so a
// chunk worker that waits for x holds nothing urgent.  (Claiming whole rows'
// bulk in row order instead makes the work grow towards the end of the
// solve, where every row has the most tiles.)
__device__ __forceinline__ void chunk_of(long t, long nb, long &K, int &c) {
  long lo = 0, hi = (nb - kD - 1) / kCT > 1 ? (nb - kD - 1) / kCT : 1;
  while (lo < hi) {
    const long mid = (lo + hi + 1) / 2;
    if (chunks_in_groups_before(mid, nb) <= t) lo = mid;
    else hi = mid - 1;
  }
  c = int(lo);
  K = kCT * (lo + 1) + kD + 1 + (t - chunks_in_groups_before(lo, nb));
}

// The first kNT threads of a streaming CTA (a 16-CTA launch has kNTS
// threads; the extra warps of a streaming CTA return at once).
__device__ __forceinline__ void work_sync() { asm volatile("bar.sync 2, 256;" ::: "memory"); }

template <typename T>
__device__ void stream_items(const Args<T> &a, SmemStream<T> &S, bool &dead, bool tail_worker) {
  __shared__ long s_item;
  __shared__ unsigned s_ready;
  const int tid = threadIdx.x, lane = tid & 31;
  const long nb = a.nb;
  const long total = tail_worker ? tail_items(nb) : chunk_items(nb);
  int *ticket = a.ctl + (tail_worker ? 2 : 1);
  const int i = tid >> 2, q = tid & 3;  // row, quarter of the tile product
  for (;;) {
    work_sync();
    if (tid == 0) s_item = atomicAdd(ticket, 1);
    work_sync();
    const long t = s_item;
    if (t >= total) return;
    long K, J0, J1;
    int c;
    if (tail_worker) {
      K = kD + 1 + t;
      c = nfull(K);
      J0 = long(c) * kCT;
      J1 = K - kD;
    } else {
      chunk_of(t, nb, K, c);
      J0 = long(c) * kCT;
      J1 = J0 + kCT;
    }
    const int ntiles = int(J1 - J0);
    // stage tiles J0, J0+1 with cp.async; element (r, cc) = L(K*64+r, J*64+cc)
    auto issue = [&](int slot, long J) {
      for (int e = tid; e < kTB * kTB; e += kNT) {
        // consecutive threads walk along A's contiguous dimension
        const int r = a.trans ? e % kTB : e / kTB, cc = a.trans ? e / kTB : e % kTB;
        const long gi = K * kTB + r, gj = J * kTB + cc;
        if (gi < a.n && gj < a.n)
          cp_async(&S.tile[slot][r][cc], a.A + lidx(a, gi, gj));
        else
          S.tile[slot][r][cc] = T(0);
      }
      cp_commit();
    };
    issue(0, J0);
    if (ntiles > 1) issue(1, J0 + 1);
    else cp_commit();  // one group per tile slot
    // which x blocks of the item are published already: one poll for the
    // whole item, then one round of loads for those x values
    if (tid < 32) {
      const int f = lane < ntiles ? ld_acquire(a.xflag + J0 + lane) : 0;
      const unsigned m = __ballot_sync(0xffffffffu, f != 0);
      if (lane == 0) s_ready = m;
    }
    work_sync();
    const unsigned ready = s_ready;
    for (int e = tid; e < ntiles * kTB; e += kNT) {
      const int tt = e / kTB;
      if ((ready >> tt) & 1u) {
        const long gj = (J0 + tt) * kTB + e % kTB;
        S.zs[tt][e % kTB] = gj < a.n ? __ldcg(a.z + zidx(a, gj)) : T(0);
      }
    }
    // Tile product: thread (i, q) takes row i and the column pairs
    // p = q + 4v (v = 0..7) as 16-byte loads, with two independent
    // accumulators (even and odd v).  With the 72-element row pitch the eight
    // lanes of a quarter-warp (rows i, i+1; q = 0..3) read eight different
    // 16-byte bank groups, so the loads are conflict-free.
    using V2 = typename V16<T>::type;
    constexpr int kVE = int(16 / sizeof(T));  // elements per 16-byte load
    constexpr int kNV = kTB / (4 * kVE);      // loads per thread and tile
    T acc = 0, acc1 = 0;
    for (int tt = 0; tt < ntiles; ++tt) {
      const long J = J0 + tt;
      cp_wait<1>();  // tile tt has landed; tile tt+1 may be in flight
      work_sync();   // ... for every thread, and tile tt-1 is no longer read
      if (tt + 2 < ntiles) issue((tt + 2) % 3, J + 2);
      else cp_commit();  // keep one group per iteration
      if (!((ready >> tt) & 1u)) {
        // x_J was not published at the claim: wait for the solver
        if (tid == 0) wait_flag(a.xflag + J, a.status, dead);
        work_sync();
        if (tid < kTB) {
          const long gj = J * kTB + tid;
          S.zs[tt][tid] = gj < a.n ? __ldcg(a.z + zidx(a, gj)) : T(0);
        }
        work_sync();
      }
      const T *row = &S.tile[tt % 3][i][0];
      const T *xv = &S.zs[tt][0];
#pragma unroll
      for (int v = 0; v < kNV; ++v) {
        const int col = (q + 4 * v) * kVE;
        const V2 l = *reinterpret_cast<const V2 *>(row + col);
        const V2 x = *reinterpret_cast<const V2 *>(xv + col);
        if constexpr (sizeof(T) == 8) {
          if (v & 1) acc1 = fma(l.y, x.y, fma(l.x, x.x, acc1));
          else acc = fma(l.y, x.y, fma(l.x, x.x, acc));
        } else {
          if (v & 1) acc1 = fma(l.w, x.w, fma(l.z, x.z, fma(l.y, x.y, fma(l.x, x.x, acc1))));
          else acc = fma(l.w, x.w, fma(l.z, x.z, fma(l.y, x.y, fma(l.x, x.x, acc))));
        }
      }
    }
    acc += acc1;
    cp_wait<0>();
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    acc += __shfl_xor_sync(0xffffffffu, acc, 2);
    if (q == 0) a.slots[(K * a.nch + c) * kTB + i] = acc;
    __threadfence();
    work_sync();
    if (tid == 0) st_release(a.sflag + K * a.nch + c, 1);
  }
}

// --------------------------------------------------------------- solver ----
// Solver cluster of CS CTAs; CTA r owns rows [r*RPC, (r+1)*RPC) of every
// block.  Per step K the critical path is: t0 = L[K,K-1] x_{K-1} for the
// owned rows -> residual exchange -> x_K = inv(L_KK) r -> x exchange.  All
// other work for step K+1 (the near tiles L[K+1, K+1-j] x_{K+1-j} for
// j = 2..kD, which only need x values already known, and the bulk slot sums)
// runs in the shadows of the two cluster barriers.
template <typename T, int CS>
struct SmemSolver {
  static constexpr int RPC = kTB / CS;
  static constexpr int kStage = (kD + 1) * RPC * kTB;  // near tiles j = 0..kD-1, then inv rows
  T stage[kPre][kStage];
  T bvals[kPre][RPC];
  T rfull[2][kTB];
  T xring[kXR][kTB];
  T nearres[2][RPC];  // shadow near-tile sums per row (one or two warps per row)
  T carry[RPC];
};

template <typename T, int CS>
__device__ void solve_chain(const Args<T> &a, SmemSolver<T, CS> &S, bool &dead) {
  constexpr int RPC = kTB / CS;
  constexpr int kStage = SmemSolver<T, CS>::kStage;
  cg::cluster_group cl = cg::this_cluster();
  const int R = int(cl.block_rank());
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long n = a.n;
  const int nb = a.nb;

  // stage K: near tile j (L[K, K-1-j]) rows at j*RPC*kTB, inv rows at kD*RPC*kTB
  auto prefetch = [&](long K) {
    if (K < nb) {
      T *st = S.stage[K % kPre];
      for (int e = tid; e < kStage; e += kNT) {
        const int which = e / (RPC * kTB), rem = e % (RPC * kTB);
        const int r = rem / kTB, cc = rem % kTB;
        const long gi = K * kTB + R * RPC + r;
        if (which < kD) {
          const long J = K - 1 - which;
          const long gj = J * kTB + cc;
          if (J >= 0 && gi < n && gj < n)
            cp_async(st + e, a.A + lidx(a, gi, gj));
          else
            st[e] = T(0);
        } else {
          cp_async(st + e, a.inv + (K * kTB + R * RPC + r) * kTB + cc);
        }
      }
      if (tid < RPC) {
        const long gi = K * kTB + R * RPC + tid;
        if (gi < n)
          cp_async(&S.bvals[K % kPre][tid], a.z + zidx(a, gi));
        else
          S.bvals[K % kPre][tid] = T(0);
      }
    }
    cp_commit();
  };
  // Measured on GB300: one warp issues at most one FP64 instruction per ~64
  // clocks and a shuffle + FP64 add step costs ~100 clocks, while the SM's
  // FP64 pipe takes a warp instruction every ~19 clocks once 4+ warps issue.
  // So FP64 work is spread one row per warp with short dependency chains.
  // rowdot: one warp, row `row` (64 entries) . v; result in every lane
  auto rowdot = [&](const T *row, const T *v) -> T {
    T s = fma(row[lane + 32], v[lane + 32], row[lane] * v[lane]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
  };
  constexpr int kWPR = (kNT / 32) / RPC;  // warps per owned row in the shadows (1 or 2)
  // lanes c < nc of the row-owner warps hold slot values of the next row
  T pend = 0;
  int pend_nc = 0;
  // warp 0 polls the slot flags of block row K2, then the row-owner warps
  // load the slot values into `pend` (used one step later)
  auto request_slots = [&](long K2) {
    pend = 0;
    pend_nc = 0;
    if (K2 >= nb) return;
    const int nc = nslots_row(K2);
    if (nc == 0) return;
    if (warp == 0 && !dead) {
      long long spins = 0;
      for (;;) {
        int ok = 1;
        for (int cc = lane; cc < nc; cc += 32) ok &= ld_acquire(a.sflag + K2 * a.nch + cc) != 0;
        if (__all_sync(0xffffffffu, ok)) break;
        if (++spins > kSpin) {
          if (lane == 0) atomicExch(a.status, 1);
          dead = true;
          break;
        }
        __nanosleep(64);
      }
    }
    __syncthreads();
    pend_nc = nc;
    // lane c of row warp w sums slots c, c+32, ... of row w (the loads
    // complete during the next step)
    if (warp < RPC) {
      T v = 0;
      for (int cc = lane; cc < nc; cc += 32) v += __ldcg(a.slots + (K2 * a.nch + cc) * kTB + R * RPC + warp);
      pend = v;
    }
  };

  for (int p = 0; p < kPre; ++p) prefetch(p);
  if (tid < RPC) S.carry[tid] = T(0);
  // bulk of rows 0 and 1 is empty (nslots_row(K) = 0 for K <= kD)
  request_slots(1);
  for (long K = 0; K < nb; ++K) {
    const int sidx = int(K % kPre);
    cp_wait<kPre - 1>();
    __syncthreads();
    const T *st = S.stage[sidx];
    // ---- critical: residual of the owned rows
    if (warp < RPC) {
      const T t0 = K >= 1 ? rowdot(st + warp * kTB, S.xring[(K - 1) % kXR]) : T(0);
      const T rr = S.bvals[sidx][warp] - S.carry[warp] - t0;
      // lane d writes the residual to CTA d
      if (lane < CS) *cl.map_shared_rank(&S.rfull[K & 1][R * RPC + warp], lane) = rr;
    }
    cluster_arrive();
    // ---- shadow 1: near tiles j = 1..kD-1 of step K+1 (x_{K-1} .. x_{K+1-kD})
    // and publishing x_{K-1} to global memory for the streamers
    if (K + 1 < nb) {
      cp_wait<kPre - 2>();
      __syncthreads();
      const T *st1 = S.stage[(K + 1) % kPre];
      // warp w: row w % RPC, near tiles j = 1 + w / RPC, 1 + w / RPC + kWPR, ...
      {
        const int r = warp % RPC, j0 = 1 + warp / RPC;
        T s0 = 0, s1 = 0;
        for (int j = j0; j < kD; j += kWPR) {
          const long J = K - j;
          if (J < 0) break;
          const T *row = st1 + (j * RPC + r) * kTB;
          const T *xv = S.xring[J % kXR];
          s0 = fma(row[lane], xv[lane], s0);
          s1 = fma(row[lane + 32], xv[lane + 32], s1);
        }
        T sum = s0 + s1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
        if (lane == 0) S.nearres[warp / RPC][r] = sum;
      }
    }
    if (R == 0 && K >= 1 && warp == RPC - 1 + (RPC < kNT / 32 ? 1 : 0)) {
      // publish x_{K-1}: the last warp writes it, fences and raises the flag
      for (int t = lane; t < kTB; t += 32) {
        const long gi = (K - 1) * kTB + t;
        if (gi < n) a.z[zidx(a, gi)] = S.xring[(K - 1) % kXR][t];
      }
      __threadfence();
      __syncwarp();
      if (lane == 0) st_release(a.xflag + K - 1, 1);
    }
    cluster_wait();
    // ---- critical: x_K rows = inv(L_KK)[rows] . rfull
    if (warp < RPC) {
      const T xk = rowdot(st + (kD * RPC + warp) * kTB, S.rfull[K & 1]);
      if (lane < CS) *cl.map_shared_rank(&S.xring[K % kXR][R * RPC + warp], lane) = xk;
    }
    cluster_arrive();
    // ---- shadow 2: refill stage K, carry for step K+1, slot loads for K+2
    __syncthreads();
    prefetch(K + kPre);
    if (warp < RPC) {
      T b = pend_nc > 0 ? pend : T(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
      if (lane == 0) {
        T nr = S.nearres[0][warp];
        if (kWPR > 1) nr += S.nearres[1][warp];
        S.carry[warp] = (K + 1 < nb) ? b + nr : T(0);
      }
    }
    request_slots(K + 2);
    cluster_wait();
  }
  // publish the last block
  if (R == 0 && warp == RPC - 1 + (RPC < kNT / 32 ? 1 : 0)) {
    for (int t = lane; t < kTB; t += 32) {
      const long gi = (nb - 1) * long(kTB) + t;
      if (gi < n) a.z[zidx(a, gi)] = S.xring[(nb - 1) % kXR][t];
    }
    __threadfence();
    __syncwarp();
    if (lane == 0) st_release(a.xflag + nb - 1, 1);
  }
  cp_wait<0>();
}

// ------------------------------------------------- solver, 16-CTA form ----
// Warps 0..3 of each solver CTA are the critical warps (warp w owns row
// R*4+w of every block), warps 4..7 the helpers.  The two exchanges of a
// step are asynchronous remote shared-memory stores (st.async) that count
// their bytes against an mbarrier in the receiving CTA (armed once per phase
// with the 64 values it expects), so only the critical warps take part in
// them, no sender waits for its stores, and no step waits on a cluster
// barrier.
// The helpers prepare step K+1 meanwhile (operand prefetch, the near tiles
// L[K+1, K-1..K-5] x, the bulk slot sums, publishing x to global memory)
// and hand the carry over through a local mbarrier.
//
// Barrier rings and why their parities cannot alias: E1 (residuals, ring 2)
// phase K completes only when every critical warp sent its step-K residual,
// which it does after waiting for phase K-2 of the same barrier.  Critical
// warp 0 re-arms a barrier for its next phase right after observing a phase
// complete; data of that next phase cannot land earlier, and if it did the
// phase would still wait for the arming arrival.  E2 (x,
// ring 4) phase m+4 needs the step-(m+4) residuals, which need the carries
// of step m+4, which the helpers produce after their last wait on phase m.
// The carry barrier (ring 2) phase K+2 is armed by the helpers only after
// E2 phase K, i.e. after the critical warps consumed phase K.
constexpr int kCS2 = 16;
constexpr int kRPC2 = kTB / kCS2;  // 4
constexpr int kSR = 4;                     // slot-sum ring depth (block rows)
constexpr int kPubWarp = kNT / 32;         // warp 8
constexpr int kLoaderWarp = kNT / 32 + 1;  // warps 9, 10: even and odd block rows
constexpr int kLoaders = 2;
static_assert(kNTS == 32 * (kLoaderWarp + kLoaders), "16-CTA solver warps");
constexpr long long kWaitCycles = 4ll << 30;

template <typename T>
struct SmemSolver2 {
  static constexpr int kStage = (kD + 1) * kRPC2 * kTB;  // near tiles j = 0..kD-1, then inv rows
  T stage[kPre][kStage];
  T bvals[kPre][kRPC2];
  T rfull[2][kTB];
  T xring[kXR][kTB];
  T carry[2][kRPC2][32];  // per-lane partial sums of the carry, added inside the critical row dot
  T slotsum[kSR][kRPC2];  // bulk sums of the owned rows, ring of kSR block rows (slot loader -> helpers)
  unsigned long long e1bar[2];
  unsigned long long e2bar[4];
  unsigned long long cready[2];
  int pub_done;    // x_0 .. x_{pub_done-1} published to global memory (publisher -> helpers)
  int slot_row[kSR];  // slotsum[i] holds block row slot_row[i] (slot loaders -> helpers)
  int slot_used;   // helpers have consumed the slot sums of rows up to slot_used (helpers -> slot loader)
};

__device__ __forceinline__ uint32_t sh_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint32_t map_rank(uint32_t a, int rank) {
  uint32_t o;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(o) : "r"(a), "r"(rank));
  return o;
}
// Remote store that completes `bytes` of the remote mbarrier's transaction
// count when it lands (no fence on the sending thread).
__device__ __forceinline__ void st_async(uint32_t a, double v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(a),
               "l"(__double_as_longlong(v)), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void st_async(uint32_t a, float v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b32 [%0], %1, [%2];" ::"r"(a),
               "r"(__float_as_uint(v)), "r"(bar)
               : "memory");
}
// One local arrival that also expects `bytes` of remote stores this phase.
__device__ __forceinline__ void arm(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sh_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void arrive_local(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void bar_init(uint32_t bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ bool bar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for the phase of parity `parity`, by a whole warp (the
// outcome is warp-uniform); on expiry records the timeout and stops waiting
// for the rest of the launch.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, int *status, bool &dead) {
  if (dead) return false;
  const long long t0 = clock64();
  for (;;) {
    if (__all_sync(0xffffffffu, bar_try(bar, parity))) return true;
    if (__shfl_sync(0xffffffffu, int(clock64() - t0 > kWaitCycles), 0)) {
      if ((threadIdx.x & 31) == 0) atomicExch(status, 1);
      dead = true;
      return false;
    }
  }
}
__device__ __forceinline__ void helper_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }
__device__ __forceinline__ int ld_acquire_cta(const int *p) {
  int v;
  asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(sh_u32(p)) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta(int *p, int v) {
  asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(sh_u32(p)), "r"(v) : "memory");
}
// Bounded wait, by a whole warp, for the shared counter *p to reach `want`.
__device__ __forceinline__ bool wait_count(const int *p, int want, int *status, bool &dead) {
  if (dead) return false;
  const long long t0 = clock64();
  for (;;) {
    if (__all_sync(0xffffffffu, ld_acquire_cta(p) >= want)) return true;
    if (__shfl_sync(0xffffffffu, int(clock64() - t0 > kWaitCycles), 0)) {
      if ((threadIdx.x & 31) == 0) atomicExch(status, 1);
      dead = true;
      return false;
    }
    __nanosleep(32);
  }
}

template <typename T>
__device__ void solve_chain2(const Args<T> &a, SmemSolver2<T> &S, bool &dead) {
  constexpr int RPC = kRPC2, CS = kCS2;
  constexpr int kStage = SmemSolver2<T>::kStage;
  cg::cluster_group cl = cg::this_cluster();
  const int R = int(cl.block_rank());
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long n = a.n;
  const int nb = a.nb;
  constexpr uint32_t kXBytes = kTB * sizeof(T);  // one exchange: 64 values from the cluster
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) bar_init(sh_u32(&S.e1bar[i]), 1);
    for (int i = 0; i < 4; ++i) bar_init(sh_u32(&S.e2bar[i]), 1);
    for (int i = 0; i < 2; ++i) bar_init(sh_u32(&S.cready[i]), 32 * (kNT / 32 - RPC));  // every helper lane
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int i = 0; i < 2; ++i) arm(sh_u32(&S.e1bar[i]), kXBytes);
    for (int i = 0; i < 4; ++i) arm(sh_u32(&S.e2bar[i]), kXBytes);
    S.pub_done = 0;
    for (int i = 0; i < kSR; ++i) S.slot_row[i] = -1;
    S.slot_used = kD;  // rows 0 .. kD have no bulk part
  }
  cl.sync();  // every barrier of the cluster is initialised before any remote arrive

  // 64-entry row . v by one warp (FP64: one row per warp keeps the chains short)
  auto rowdot = [&](const T *row, const T *v) -> T {
    T s = fma(row[lane + 32], v[lane + 32], row[lane] * v[lane]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return s;
  };

  if (warp < RPC) {
    // ---------------- critical warp: row R*RPC + w of every block
    const int w = warp;
    for (long K = 0; K < nb; ++K) {
      bar_wait(sh_u32(&S.cready[K & 1]), uint32_t((K >> 1) & 1), a.status, dead);
      const T *st = S.stage[K % kPre];
      // carry + L[K,K-1] x_{K-1}: the helpers' per-lane partials start the
      // lane sums, so one tree reduces both
      T s = S.carry[K & 1][w][lane];
      if (K >= 1) {
        bar_wait(sh_u32(&S.e2bar[(K - 1) & 3]), uint32_t(((K - 1) >> 2) & 1), a.status, dead);
        if (w == 0 && lane == 0) arm(sh_u32(&S.e2bar[(K - 1) & 3]), kXBytes);  // for step K+3
        const T *row = st + w * kTB, *xv = S.xring[(K - 1) % kXR];
        s = fma(row[lane + 32], xv[lane + 32], fma(row[lane], xv[lane], s));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      const T rr = S.bvals[K % kPre][w] - s;
      if (lane < CS)  // lane d hands the residual to CTA d
        st_async(map_rank(sh_u32(&S.rfull[K & 1][R * RPC + w]), lane), rr, map_rank(sh_u32(&S.e1bar[K & 1]), lane));
      bar_wait(sh_u32(&S.e1bar[K & 1]), uint32_t((K >> 1) & 1), a.status, dead);
      if (w == 0 && lane == 0) arm(sh_u32(&S.e1bar[K & 1]), kXBytes);  // for step K+2
      const T xk = rowdot(st + (kD * RPC + w) * kTB, S.rfull[K & 1]);
      if (lane < CS)
        st_async(map_rank(sh_u32(&S.xring[K % kXR][R * RPC + w]), lane), xk, map_rank(sh_u32(&S.e2bar[K & 3]), lane));
    }
  } else if (warp < kNT / 32) {
    // ---------------- helper warps: warp RPC + h prepares row h's carry
    const int h = warp - RPC;
    const int ht = tid - RPC * 32;  // 0 .. 127
    auto prefetch = [&](long K) {
      if (K < nb && a.vec16) {
        // helper warp h copies row h of each near tile and of the inverse,
        // 16 bytes per lane
        constexpr int kPer = 16 / int(sizeof(T)), kChunks = kTB / kPer;
        T *st = S.stage[K % kPre];
        const long gi = K * kTB + R * RPC + h;
        if (lane < kChunks) {
          for (int which = 0; which <= kD; ++which) {
            T *dst = st + (which * RPC + h) * kTB + lane * kPer;
            if (which == kD) {
              cp_async16(dst, a.inv + (K * kTB + R * RPC + h) * kTB + lane * kPer);
            } else {
              const long J = K - 1 - which;
              if (J >= 0 && gi < n)
                cp_async16(dst, a.A + gi * a.lda + J * kTB + lane * kPer);
              else
                *reinterpret_cast<uint4 *>(dst) = make_uint4(0u, 0u, 0u, 0u);
            }
          }
        }
      } else if (K < nb) {
        T *st = S.stage[K % kPre];
        for (int e = ht; e < kStage; e += 32 * (kNT / 32 - RPC)) {
          const int which = e / (RPC * kTB), rem = e % (RPC * kTB);
          const int r = rem / kTB, cc = rem % kTB;
          const long gi = K * kTB + R * RPC + r;
          if (which < kD) {
            const long J = K - 1 - which;
            const long gj = J * kTB + cc;
            if (J >= 0 && gi < n && gj < n)
              cp_async(st + e, a.A + lidx(a, gi, gj));
            else
              st[e] = T(0);
          } else {
            cp_async(st + e, a.inv + (K * kTB + R * RPC + r) * kTB + cc);
          }
        }
      }
      if (K < nb && ht < RPC) {
        const long gi = K * kTB + R * RPC + ht;
        if (gi < n)
          cp_async(&S.bvals[K % kPre][ht], a.z + zidx(a, gi));
        else
          S.bvals[K % kPre][ht] = T(0);
      }
      cp_commit();
    };
    for (int p = 0; p < kPre; ++p) prefetch(p);
    cp_wait<kPre - 1>();
    helper_sync();
    S.carry[0][h][lane] = T(0);
    arrive_local(sh_u32(&S.cready[0]));
    // Iteration T1 prepares the carry of step T1.  It starts when x_{T1-2}
    // is exchanged: the stage of step T1-2 is then free for step T1-2+kPre;
    // the carry is the near tiles up to x_{T1-2} plus the bulk sums of row
    // T1, which the slot loader has summed into slotsum ahead of time.
    for (long T1 = 1; T1 < nb; ++T1) {
      if (T1 >= 2) {
        bar_wait(sh_u32(&S.e2bar[(T1 - 2) & 3]), uint32_t(((T1 - 2) >> 2) & 1), a.status, dead);
        prefetch(T1 - 2 + kPre);
      } else {
        cp_commit();  // one group per iteration
      }
      // The publisher must keep within three steps: the e2bar ring (4) and
      // the x ring (8) it reads stay unaliased while step T1 waits for it.
      wait_count(&S.pub_done, int(T1 - 3), a.status, dead);
      // groups so far: stages 0..kPre-1, one empty, then stage g-1 in group
      // g; stage T1 is complete once at most two groups are outstanding
      cp_wait<kPre - 2>();
      helper_sync();
      // every helper has finished iteration T1-1: slot sums up to row T1-1 consumed
      if (h == 0 && lane == 0 && T1 - 1 > kD) st_release_cta(&S.slot_used, int(T1 - 1));
      const T *st = S.stage[T1 % kPre];
      T s0 = T(0), s1 = T(0);
      for (int j = 1; j < kD; ++j) {
        const long J = T1 - 1 - j;
        if (J < 0) break;
        const T *row = st + (j * RPC + h) * kTB;
        const T *xv = S.xring[J % kXR];
        s0 = fma(row[lane], xv[lane], s0);
        s1 = fma(row[lane + 32], xv[lane + 32], s1);
      }
      T bulk = T(0);
      if (nslots_row(T1) > 0) {
        wait_count(&S.slot_row[T1 % kSR], int(T1), a.status, dead);
        bulk = S.slotsum[T1 % kSR][h];
      }
      S.carry[T1 & 1][h][lane] = (s0 + s1) + (lane == 0 ? bulk : T(0));
      arrive_local(sh_u32(&S.cready[T1 & 1]));
    }
    cp_wait<0>();
  } else if (warp == kPubWarp) {
    // ---------------- publisher: x_m to global memory and its release flag,
    // by the CTA m % CS, as soon as x_m is exchanged
    for (long m = 0; m < nb; ++m) {
      bar_wait(sh_u32(&S.e2bar[m & 3]), uint32_t((m >> 2) & 1), a.status, dead);
      if (m % CS == R) {
        for (int t = lane; t < kTB; t += 32) {
          const long gi = m * kTB + t;
          if (gi < n) a.z[zidx(a, gi)] = S.xring[m % kXR][t];
        }
        __threadfence();
        __syncwarp();
        if (lane == 0) st_release(a.xflag + m, 1);
      }
      __syncwarp();
      if (lane == 0) st_release_cta(&S.pub_done, int(m + 1));
    }
  } else if (warp < kLoaderWarp + kLoaders) {
    // ---------------- slot loaders: loader L takes block rows m = kD+1+L,
    // kD+1+L+kLoaders, ...: waits for the streamers' slots, sums the owned
    // rows' slots (lane l: row l / 8, slots l % 8 + 8u in slot order, a fixed
    // tree over u, then a fixed tree over the eight lanes of the row) and
    // hands the sums to the helpers through slotsum.
    const int L = warp - kLoaderWarp;
    const int r = lane >> 3, q = lane & 7;
    // one poll of row m's slot flags; true when all are set
    auto flags_ready = [&](long m) -> bool {
      const int nc = nslots_row(m);
      int ok = 1;
      for (int cc = lane; cc < nc; cc += 32) ok &= ld_acquire(a.sflag + m * a.nch + cc) != 0;
      return __all_sync(0xffffffffu, ok) != 0;
    };
    auto wait_flags = [&](long m, bool seen) {
      if (dead || seen) return;
      const long long t0 = clock64();
      while (!flags_ready(m)) {
        if (__shfl_sync(0xffffffffu, int(clock64() - t0 > kWaitCycles), 0)) {
          if (lane == 0) atomicExch(a.status, 1);
          dead = true;
          return;
        }
      }
    };
    // slots c0 + 8u (u = 0..7) of this lane, summed by a fixed tree; the
    // upper half is empty when the row has at most c0 + 32 slots
    const T *sl_base = a.slots + R * RPC + r;
    auto batch = [&](long m, int nc, int c0) -> T {
      const T *sl = sl_base + (m * a.nch) * kTB;
      T w[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) w[u] = c0 + q + 8 * u < nc ? __ldcg(sl + long(c0 + q + 8 * u) * kTB) : T(0);
      const T lo = (w[0] + w[1]) + (w[2] + w[3]);
      return nc <= c0 + 32 ? lo : lo + ((w[4] + w[5]) + (w[6] + w[7]));
    };
    bool next_seen = false;
    for (long m = kD + 1 + L; m < nb; m += kLoaders) {
      const int nc = nslots_row(m);
      wait_count(&S.slot_used, int(m - kSR), a.status, dead);  // row m - kSR consumed
      wait_flags(m, next_seen);
      // the first batch of loads in flight while the flags of this loader's
      // next row are polled once
      const T *sl = sl_base + (m * a.nch) * kTB;
      T w[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) w[u] = q + 8 * u < nc ? __ldcg(sl + long(q + 8 * u) * kTB) : T(0);
      next_seen = m + kLoaders < nb && !dead && flags_ready(m + kLoaders);
      T v = (w[0] + w[1]) + (w[2] + w[3]);
      if (nc > 32) v += (w[4] + w[5]) + (w[6] + w[7]);
      for (int c0 = 64; c0 < nc; c0 += 64) v += batch(m, nc, c0);
      v += __shfl_xor_sync(0xffffffffu, v, 4);
      v += __shfl_xor_sync(0xffffffffu, v, 2);
      v += __shfl_xor_sync(0xffffffffu, v, 1);
      if (q == 0) S.slotsum[m % kSR][r] = v;
      __syncwarp();
      __threadfence_block();
      if (lane == 0) st_release_cta(&S.slot_row[m % kSR], int(m));
    }
  }
  cl.sync();  // no CTA leaves while a peer may still write into its shared memory
}

template <typename T, int CS>
__global__ void __launch_bounds__(kNTS, 1) trsv_cluster_kernel(Args<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cg::cluster_group cl = cg::this_cluster();
  __shared__ int s_role;
  // role: rank 0 of each cluster tries to claim the solver role
  if (threadIdx.x == 0) s_role = 0;
  if (cl.block_rank() == 0 && threadIdx.x == 0) {
    s_role = atomicCAS(a.ctl, 0, 1) == 0 ? 1 : 0;
    atomicAdd(a.ctl + 3, 1);  // this cluster is resident
  }
  cl.sync();
  const int role = *cl.map_shared_rank(&s_role, 0);
  cl.sync();
  bool dead = false;
  if (role == 1) {
    if constexpr (CS == kCS2)
      solve_chain2<T>(a, *reinterpret_cast<SmemSolver2<T> *>(smem_raw), dead);
    else
      solve_chain<T, CS>(a, *reinterpret_cast<SmemSolver<T, CS> *>(smem_raw), dead);
  } else if (threadIdx.x < kNT) {  // a 16-CTA launch's extra warps have no streaming work
    stream_items<T>(a, *reinterpret_cast<SmemStream<T> *>(smem_raw), dead, int(cl.block_rank()) < kTailCTAs);
  }
}

// Extra streaming CTAs, launched on a side stream beside the clustered
// launch to use the SMs that its clusters leave free (16-CTA clusters
// occupy whole GPC partitions; the remainder of each GPC would idle).  They
// take chunk items only, and only once every cluster of the clustered launch
// is resident (each counts itself in ctl[3] as it starts).  The clustered
// launch can then finish all the work by itself, so the extra CTAs only
// speed it up and can never hold an SM that a cluster still needs: a CTA
// that finds the clusters incomplete waits at most kExtraWaitNs and leaves.
// Two of them fit on a free SM; a clustered CTA takes more shared memory
// than is left next to one, so none of them shares an SM with a solver CTA.
constexpr unsigned long long kExtraWaitNs = 20000;
template <typename T>
__global__ void __launch_bounds__(kNT, 1) trsv_extra_stream_kernel(Args<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_go;
  if (threadIdx.x == 0) {
    unsigned long long t0, t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    int go = ld_acquire(a.ctl + 3) >= a.nclusters;
    while (!go) {
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      if (t - t0 > kExtraWaitNs) break;
      __nanosleep(256);
      go = ld_acquire(a.ctl + 3) >= a.nclusters;
    }
    s_go = go;
  }
  __syncthreads();
  if (!s_go) return;
  bool dead = false;
  stream_items<T>(a, *reinterpret_cast<SmemStream<T> *>(smem_raw), dead, false);
}

// ------------------------------------------------- diagonal-block inverse --
// inv[K] = inverse of the effective lower-triangular diagonal block L_KK
// (unit diagonal when `unit`; rows/columns beyond n are the identity).
// Column c of the inverse is y with L y = e_c: y_c = 1/L_cc,
// y_i = -(sum_{j=c}^{i-1} L_ij y_j) * (1/L_ii); four lanes share a column.
// The reciprocals of the diagonal are formed once (64 divisions per block):
// an FP64 division per element is far too slow on this FP64 pipe.
template <typename T>
__global__ void __launch_bounds__(kNT) trsv_inverse_kernel(Args<T> a) {
  __shared__ T L[kTB][kTB + 1];
  __shared__ T Y[kTB][kTB + 1];  // Y[i][c]
  __shared__ T rd[kTB];
  const long K = blockIdx.x;
  const int tid = threadIdx.x;
  for (int e = tid; e < kTB * kTB; e += kNT) {
    const int r = a.trans ? e % kTB : e / kTB, cc = a.trans ? e / kTB : e % kTB;
    const long gi = K * kTB + r, gj = K * kTB + cc;
    T v;
    if (gi < a.n && gj < a.n)
      v = cc <= r ? a.A[lidx(a, gi, gj)] : T(0);
    else
      v = r == cc ? T(1) : T(0);
    if (r == cc && (a.unit || gi >= a.n)) v = T(1);
    L[r][cc] = v;
    Y[r][cc] = T(0);
  }
  __syncthreads();
  if (tid < kTB) rd[tid] = T(1) / L[tid][tid];
  __syncthreads();
  // Blocked inverse: 16x16 leaves by substitution, then 32x32 and 64x64 by
  // inv([A 0; B C]) = [inv(A) 0; -inv(C) B inv(A), inv(C)], the products
  // taking the triangles into account.  The dependency chains are 16 steps
  // instead of 64; the FMA count stays n^3/6.  The strictly upper 32x32
  // block of L (zeros, never read) holds the products' scratch:
  // W(i, j) = L[i][32 + j].
  {
    // leaves: four 16x16 blocks, 64 threads each, 4 lanes per column
    const int o = (tid >> 6) * 16, c = (tid & 63) >> 2, q = tid & 3;
    const unsigned mask = 0xfu << ((threadIdx.x & 31) & ~3);
    if (q == 0) Y[o + c][o + c] = rd[o + c];
    __syncwarp(mask);
    for (int i = c + 1; i < 16; ++i) {
      T s = 0;
      for (int j = c + q; j < i; j += 4) s = fma(L[o + i][o + j], Y[o + j][o + c], s);
      s += __shfl_xor_sync(mask, s, 1);
      s += __shfl_xor_sync(mask, s, 2);
      if (q == 0) Y[o + i][o + c] = -s * rd[o + i];
      __syncwarp(mask);
    }
  }
  __syncthreads();
  static_assert(kNT == 256 && kTB == 64, "the stages below map 8 warps onto 64x64 blocks");
  const int w = tid >> 5, lane = tid & 31;
  // 32x32 blocks p = 0, 1 at P = 32p (lanes 0-15: P = 0, lanes 16-31: P = 32):
  //   W = L[P+16.., P..] inv(A)     W(i, j) = sum_{k=j..15} L[P+16+i][P+k] Y[P+k][P+j]
  {
    const int P = (lane >> 4) * 32, i = lane & 15;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int j = h ? 15 - w : w;
      T s = 0;
      for (int k = j; k < 16; ++k) s = fma(L[P + 16 + i][P + k], Y[P + k][P + j], s);
      L[(P >> 1) + i][32 + j] = s;
    }
  }
  __syncthreads();
  //   Y[P+16+i][P+j] = - sum_{k=0..i} Y[P+16+i][P+16+k] W(k, j)
  {
    const int P = (lane >> 4) * 32, j = lane & 15;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int i = h ? 15 - w : w;
      T s = 0;
      for (int k = 0; k <= i; ++k) s = fma(Y[P + 16 + i][P + 16 + k], L[(P >> 1) + k][32 + j], s);
      Y[P + 16 + i][P + j] = -s;
    }
  }
  __syncthreads();
  // 64x64: W = L[32.., 0..31] inv(A32)   W(i, j) = sum_{k=j..31} L[32+i][k] Y[k][j]
  // (warp w: columns w, 31-w, 8+w, 23-w; lane i)
  {
    const int i = lane;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int j = (h & 1) ? 31 - (w + 8 * (h >> 1)) : w + 8 * (h >> 1);
      T s = 0;
      for (int k = j; k < 32; ++k) s = fma(L[32 + i][k], Y[k][j], s);
      L[i][32 + j] = s;
    }
  }
  __syncthreads();
  //   Y[32+i][j] = - sum_{k=0..i} Y[32+i][32+k] W(k, j)   (warp w: rows w, 31-w, 8+w, 23-w; lane j)
  {
    const int j = lane;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      const int i = (h & 1) ? 31 - (w + 8 * (h >> 1)) : w + 8 * (h >> 1);
      T s = 0;
      for (int k = 0; k <= i; ++k) s = fma(Y[32 + i][32 + k], L[k][32 + j], s);
      Y[32 + i][j] = -s;
    }
  }
  __syncthreads();
  T *out = const_cast<T *>(a.inv) + K * kTB * kTB;
  for (int e = tid; e < kTB * kTB; e += kNT) out[e] = Y[e / kTB][e % kTB];
}

}  // namespace tc

template <typename T, int CS>
size_t trsv_cluster_smem() {
  const size_t a = CS == tc::kCS2 ? sizeof(tc::SmemSolver2<T>) : sizeof(tc::SmemSolver<T, CS>);
  const size_t b = sizeof(tc::SmemStream<T>);
  size_t s = a > b ? a : b;
  // more than half an SM's shared memory, and more than what is left next to
  // an extra streaming CTA, so a solver CTA never shares its SM (and FP64
  // pipe) with a streaming CTA of either launch
  return s > size_t(130) * 1024 ? s : size_t(130) * 1024;
}

template <typename T, int CS>
static int max_clusters(cudaLaunchConfig_t &cfg, cudaLaunchAttribute *attr) {
  auto kern = tc::trsv_cluster_kernel<T, CS>;
  const size_t smem = trsv_cluster_smem<T, CS>();
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (CS > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  attr[0].val.clusterDim.x = CS;
  cfg.dynamicSmemBytes = smem;
  cfg.blockDim = dim3(CS == tc::kCS2 ? tc::kNTS : tc::kNT);
  cfg.gridDim = dim3(CS * 32);
  int m = 0;
  if (cudaOccupancyMaxActiveClusters(&m, kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return m;
}

// Returns false when the device cannot co-schedule the clusters this needs
// (the caller then uses the single-kernel path in trsv.cu).
template <typename T>
bool trsv_cluster(bool upper, bool trans, bool unit, long n, const T *A, long lda, T *x) {
  using namespace tc;
  Context &c = ctx();
  const int nb = int(ceil_div(n, kTB));
  const int nch = nslots_row(nb - 1) > 0 ? nslots_row(nb - 1) : 1;
  // cluster size: 16 where two or more such clusters fit, else 8 (cached per device)
  static int cs_cache[64] = {0};
  static int mc_cache[64] = {0};
  static std::once_flag probed[64];
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 8;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kNT);
  cfg.stream = c.stream;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const int dev = c.device < 64 ? c.device : 63;
  std::call_once(probed[dev], [&] {
    const int m16 = max_clusters<T, 16>(cfg, attr);
    const int m8 = max_clusters<T, 8>(cfg, attr);
    if (m16 >= 4) {
      cs_cache[dev] = 16;
      mc_cache[dev] = m16;
    } else {
      cs_cache[dev] = 8;
      mc_cache[dev] = m8;
    }
  });
  const int CS = cs_cache[dev];
  const long maxc = mc_cache[dev];
  if (maxc < 1) return false;
  const long items = chunk_items(nb) + tail_items(nb);
  long clusters = 1 + ceil_div(items, CS);
  if (clusters > maxc) clusters = maxc;
  if (items > 0 && clusters < 2) return false;  // the solver needs streamers
  attr[0].val.clusterDim.x = CS;
  cfg.blockDim = dim3(CS == kCS2 ? kNTS : kNT);
  cfg.dynamicSmemBytes = CS == 16 ? trsv_cluster_smem<T, 16>() : trsv_cluster_smem<T, 8>();
  cfg.gridDim = dim3(unsigned(clusters * CS));

  // scratch: inverses, slots, flags, control words
  const size_t inv_b = (size_t(nb) * kTB * kTB * sizeof(T) + 255) & ~size_t(255);
  const size_t slot_b = (size_t(nb) * nch * kTB * sizeof(T) + 255) & ~size_t(255);
  const size_t flag_b = (size_t(nb) * (1 + nch) + 4) * 4;
  char *base = static_cast<char *>(scratch(inv_b + slot_b + flag_b));
  Args<T> a;
  a.n = n;
  a.A = A;
  a.lda = lda;
  a.z = x;
  a.inv = reinterpret_cast<T *>(base);
  a.slots = reinterpret_cast<T *>(base + inv_b);
  a.xflag = reinterpret_cast<int *>(base + inv_b + slot_b);
  a.sflag = a.xflag + nb;
  a.ctl = a.sflag + size_t(nb) * nch;
  a.status = device_status_word();
  a.nb = nb;
  a.nch = nch;
  a.nclusters = int(clusters);
  a.rev = upper != trans;
  a.trans = trans;
  a.unit = unit;
  a.vec16 = !a.rev && !trans && (lda * long(sizeof(T))) % 16 == 0 && aligned16(A);
  EXB_CUDA(cudaMemsetAsync(a.xflag, 0, flag_b, c.stream));
  trsv_inverse_kernel<T><<<nb, kNT, 0, c.stream>>>(a);
  EXB_LAUNCH("trsv inverse kernel");
  // SMs the clustered launch leaves free, when it is at its size limit, times
  // the extra CTAs that fit on one of them (two: one computes while the other
  // waits on memory)
  const long free_sms = clusters == maxc ? long(c.sm_count) - clusters * CS : 0;
  long extra = 0;
  if (free_sms > 0) {
    const size_t esmem = sizeof(SmemStream<T>);
    static std::once_flag attr_set[64];
    std::call_once(attr_set[dev], [&] {
      EXB_CUDA(cudaFuncSetAttribute(trsv_extra_stream_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    int(esmem)));
    });
    extra = free_sms * resident_per_sm(reinterpret_cast<const void *>(trsv_extra_stream_kernel<T>), kNT, esmem);
  }
  const bool use_extra = extra > 0 && chunk_items(nb) > 0;
  if (use_extra) {
    if (!c.side) {
      EXB_CUDA(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking));
      EXB_CUDA(cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming));
      EXB_CUDA(cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming));
    }
    // the side stream starts where the clustered launch starts
    EXB_CUDA(cudaEventRecord(c.fork, c.stream));
    EXB_CUDA(cudaStreamWaitEvent(c.side, c.fork, 0));
  }
  if (CS == 16)
    EXB_CUDA(cudaLaunchKernelEx(&cfg, trsv_cluster_kernel<T, 16>, a));
  else
    EXB_CUDA(cudaLaunchKernelEx(&cfg, trsv_cluster_kernel<T, 8>, a));
  count_launch(2);
  if (use_extra) {
    trsv_extra_stream_kernel<T><<<unsigned(extra), kNT, sizeof(SmemStream<T>), c.side>>>(a);
    EXB_LAUNCH("trsv extra streaming kernel");
    count_launch();
    EXB_CUDA(cudaEventRecord(c.join, c.side));
    EXB_CUDA(cudaStreamWaitEvent(c.stream, c.join, 0));
  }
  c.status_pending = true;
  return true;
}

template bool trsv_cluster<float>(bool, bool, bool, long, const float *, long, float *);
template bool trsv_cluster<double>(bool, bool, bool, long, const double *, long, double *);

}  // namespace l2
}  // namespace exb
