// Triangular solve (src/level2/trsv.py:10-52) as blocked substitution in one
// persistent launch.
//
// All four Uplo x Trans cases are mapped to a lower-triangular solve
// L z = b over "effective" indices: with c(k) = rev ? n-1-k : k,
//   L(i, j) = trans ? A[c(j)][c(i)] : A[c(i)][c(j)],  rev = upper != trans,
// and x[c(i)] = z[i].  Effective block rows of kB rows are claimed in
// increasing order through an atomic ticket, so every block a CTA waits on
// was claimed earlier by a running CTA.  A CTA owning block row K streams
// the tiles L[K, J] (J < K) through shared memory, waits for block J's
// ready flag before using x_J, then solves the diagonal block in shared
// memory (working precision: FP64 for dtrsv) and publishes x_K with a
// release flag.  Every wait is bounded: on expiry the CTA records a timeout
// in the device status word and stops, and the host reports
// EXOBLAS_TIMEOUT.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {
namespace l2 {

constexpr int kB = 64;
constexpr int kTThreads = 256;
constexpr long long kSpinLimit = 1ll << 24;  // ~ seconds with the back-off below
constexpr long kClusterMinN = 192;            // from here on the clustered solver is used

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <typename T>
__global__ void __launch_bounds__(kTThreads)
    trsv_kernel(long n, const T *__restrict__ A, long lda, T *z, bool rev, bool trans, bool unit, int *flags,
                int *ticket, int *status) {
  __shared__ T tile[kB][kB + 1];  // tile[i][j] = L(K*kB + i, J*kB + j)
  __shared__ T zs[kB];            // x_J, then the block's right-hand side
  __shared__ int s_k, s_abort;
  const int tid = threadIdx.x;
  const long nb = ceil_div(n, kB);
  auto cidx = [&](long k) { return rev ? n - 1 - k : k; };
  // loads tile L[K, J] into shared memory; A is read along its rows
  auto load_tile = [&](long K, long J) {
    for (int t = tid; t < kB * kB; t += kTThreads) {
      const int r = t / kB, c = t % kB;  // r, c index A-contiguous order below
      // choose (i, j) so that consecutive threads read consecutive A columns
      int i, j;
      if (!trans) {
        i = r;
        j = c;
      } else {
        i = c;
        j = r;
      }
      const long gi = K * kB + i, gj = J * kB + j;
      T v = T(0);
      if (gi < n && gj < n && gj <= gi) {
        const long ar = trans ? cidx(gj) : cidx(gi), ac = trans ? cidx(gi) : cidx(gj);
        v = A[ar * lda + ac];
      }
      tile[i][j] = v;
    }
  };
  if (tid == 0) s_abort = 0;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_k = atomicAdd(ticket, 1);
    __syncthreads();
    const long K = s_k;
    if (K >= nb || s_abort) break;
    // row sums of L[K, 0:K] z[0:K]; thread owns row i = tid / 4, quarter q
    const int i = tid >> 2, q = tid & 3;
    T acc = 0;
    for (long J = 0; J < K; ++J) {
      __syncthreads();
      load_tile(K, J);
      if (tid == 0) {
        long long spins = 0;
        while (ld_acquire(flags + J) == 0) {
          if (++spins > kSpinLimit) {
            s_abort = 1;
            atomicExch(status, 1);
            break;
          }
          __nanosleep(64);
        }
      }
      __syncthreads();
      if (s_abort) break;
      if (tid < kB) {
        const long gj = J * kB + tid;
        zs[tid] = gj < n ? __ldcg(z + cidx(gj)) : T(0);
      }
      __syncthreads();
#pragma unroll
      for (int jj = 0; jj < kB / 4; ++jj) {
        const int j = q * (kB / 4) + jj;
        acc = fma(tile[i][j], zs[j], acc);
      }
    }
    if (s_abort) break;
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    acc += __shfl_xor_sync(0xffffffffu, acc, 2);
    __syncthreads();
    load_tile(K, K);
    if (q == 0) {
      const long gi = K * kB + i;
      zs[i] = gi < n ? __ldcg(z + cidx(gi)) - acc : T(0);
    }
    __syncthreads();
    // diagonal block: forward substitution by one warp, lane owns rows
    // lane and lane + 32; trsv.py:31-36 divides by the diagonal.
    if (tid < 32) {
      const int l = tid;
      T r0 = zs[l], r1 = zs[l + 32];
      const long rows = n - K * kB < kB ? n - K * kB : kB;
      for (int j = 0; j < rows; ++j) {
        T xj;
        if (j < 32) {
          T mine = r0;
          if (l == j && !unit) mine = r0 / tile[j][j];
          xj = __shfl_sync(0xffffffffu, mine, j);
          if (l == j) r0 = xj;
          if (l > j) r0 = fma(-tile[l][j], xj, r0);
          r1 = fma(-tile[l + 32][j], xj, r1);
        } else {
          T mine = r1;
          if (l == j - 32 && !unit) mine = r1 / tile[j][j];
          xj = __shfl_sync(0xffffffffu, mine, j - 32);
          if (l == j - 32) r1 = xj;
          if (l > j - 32) r1 = fma(-tile[l + 32][j], xj, r1);
        }
      }
      const long g0 = K * kB + l, g1 = K * kB + l + 32;
      if (g0 < n) z[cidx(g0)] = r0;
      if (g1 < n) z[cidx(g1)] = r1;
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      st_release(flags + K, 1);
    }
  }
}

template <typename T>
bool trsv_cluster(bool upper, bool trans, bool unit, long n, const T *A, long lda, T *x);

template <typename T>
void trsv(bool upper, bool trans, bool unit, long n, const T *A, long lda, T *x, long incx) {
  if (n <= 0) return;
  // large contiguous solves: the clustered solver (trsv_cluster.cu)
  if (incx == 1 && n >= kClusterMinN && trsv_cluster<T>(upper, trans, unit, n, A, lda, x)) return;
  Context &c = ctx();
  const long nb = ceil_div(n, kB);
  // scratch: contiguous z (only when x is strided), nb flags, ticket
  const bool inplace = incx == 1;
  const size_t zbytes = inplace ? 0 : (size_t(n) * sizeof(T) + 255) & ~size_t(255);
  char *base = static_cast<char *>(scratch(zbytes + size_t(nb + 1) * 4));
  T *z = inplace ? x : reinterpret_cast<T *>(base);
  int *flags = reinterpret_cast<int *>(base + zbytes);
  int *ticket = flags + nb;
  int *status = device_status_word();
  EXB_CUDA(cudaMemsetAsync(flags, 0, size_t(nb + 1) * 4, c.stream));
  if (!inplace) l1::copy<T>(n, x, incx, z, 1);
  int blocks = int(nb < grid_cap(4) ? nb : grid_cap(4));
  trsv_kernel<T><<<blocks, kTThreads, 0, c.stream>>>(n, A, lda, z, upper != trans, trans, unit, flags, ticket, status);
  EXB_LAUNCH("trsv kernel");
  count_launch();
  if (!inplace) l1::copy<T>(n, z, 1, x, incx);
  // the timeout flag is read at the call's final synchronisation (blocking
  // mode) or by exoblas_synchronize()
  c.status_pending = true;
}

template void trsv<float>(bool, bool, bool, long, const float *, long, float *, long);
template void trsv<double>(bool, bool, bool, long, const double *, long, double *, long);

}  // namespace l2
}  // namespace exb
