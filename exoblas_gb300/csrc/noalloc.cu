// exoblas_sgemv_noalloc: exo_sgemv for callers that cannot allocate device
// memory.  Everything it needs beyond the caller's own operands lives in one
// fixed array compiled into this library (g_noalloc_scratch below); the call
// never asks the CUDA runtime, the driver or any other library for memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or forbidden,
// such as a plugin or custom-call handler inside a framework whose allocator
// owns all device memory and hands it only pre-sized buffers, or a
// latency-critical loop that must not block in the driver's allocator.
//
// Scratch: kNoAllocScratchBytes (4 MiB) of static device memory, held on
// every GPU that loads this library until the process exits.  A Trans call
// keeps its per-chunk column partial sums there (chunks x N floats, at least
// one chunk), and any call with a strided or unaligned x keeps a packed copy
// of x there (length of x floats); calls whose needs exceed the array are
// rejected with EXOBLAS_INVALID_VALUE before any work is queued.  Nothing in
// the array has to start at zero: every partial sum and the packed x are
// written before they are read.  All calls share the one array and it keeps
// the previous call's contents, so calls whose work overlaps on the GPU
// (different streams, or different host threads) race: serialise them.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture begins on that device.
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

#include "common.cuh"
#include "gemv_kernels.cuh"
#include "runtime.h"

namespace exb {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDev = 64;
struct DevInfo {
  std::atomic<bool> ready{false};
  unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch
  int sm_count = 0;
};
DevInfo g_dev[kMaxDev];
std::mutex g_setup_mutex;

// Once per device, with that device current.
DevInfo &device_setup() {
  int dev = 0;
  EXB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDev) fail(EXOBLAS_NOT_SUPPORTED, "device index out of range");
  DevInfo &d = g_dev[dev];
  if (d.ready.load(std::memory_order_acquire)) return d;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!d.ready.load(std::memory_order_relaxed)) {
    void *p = nullptr;
    // host code sees g_noalloc_scratch only as a stand-in symbol: its device
    // address comes from the runtime
    EXB_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    int sms = 0;
    EXB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    d.scratch = static_cast<unsigned char *>(p);
    d.sm_count = sms;
    d.ready.store(true, std::memory_order_release);
  }
  return d;
}

// Device or managed memory that the current device owns (a pointer into
// another GPU's memory is refused rather than read as a peer access).
bool on_device(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeDevice) return a.device == dev;
  return a.type == cudaMemoryTypeManaged;
}

// y = beta * y, or y = 0 without reading y when beta == 0: what exo_sgemv's
// scal does when x is empty (scal.py:9-19).
__global__ void beta_scale_kernel(long n, float beta, float *y, long incy) {
  for (long i = blockIdx.x * long(blockDim.x) + threadIdx.x; i < n; i += long(gridDim.x) * blockDim.x) {
    float &v = y[i * incy];
    v = beta == 0.0f ? 0.0f : beta * v;
  }
}

size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

// Same arithmetic and kernels as exo_sgemv (src/level2/gemv.py:10-22),
// launched on the caller's stream without waiting.  Column-major calls are
// taken exactly when exo_sgemv takes them (exoblas_set_column_major).
static void sgemv_noalloc(int order, int TransA, int M, int N, float alpha, const float *A, int lda, const float *X,
                          int incX, float beta, float *Y, int incY, cudaStream_t stream) {
  using namespace l2;
  if (order == kColMajor && column_major_enabled()) {
    // as exo_sgemv: a column-major M x N matrix is the row-major N x M
    // matrix of its transpose
    order = kRowMajor;
    TransA = TransA == kNoTrans ? kTrans : kNoTrans;
    const int t = M;
    M = N;
    N = t;
  }
  if (order != kRowMajor) fail(EXOBLAS_UNSUPPORTED_ORDER, "Order must be CblasRowMajor");
  if (M < 0 || N < 0) fail(EXOBLAS_INVALID_VALUE, "M < 0 or N < 0");
  const bool trans = TransA != kNoTrans;
  const long rows = M, cols = N;
  const long xlen = trans ? rows : cols, ylen = trans ? cols : rows;
  if (ylen == 0) return;
  if (incY == 0) fail(EXOBLAS_INVALID_VALUE, "incY == 0");
  if (!Y) fail(EXOBLAS_INVALID_VALUE, "NULL operand");
  if (incY < 0) Y = Y + (1 - ylen) * long(incY);
  DevInfo &d = device_setup();
  if (xlen == 0) {
    // y = beta * y (gemv.py:13-14); alpha is not used, so a NaN alpha does
    // not reach y, as in exo_sgemv
    if (!on_device(Y)) fail(EXOBLAS_INVALID_VALUE, "exoblas_sgemv_noalloc takes device pointers only");
    long blocks = ceil_div(ylen, kThreads);
    if (blocks > long(d.sm_count) * 4) blocks = long(d.sm_count) * 4;
    beta_scale_kernel<<<int(blocks), kThreads, 0, stream>>>(ylen, beta, Y, incY);
    EXB_LAUNCH("beta scale kernel");
    count_launch();
    return;
  }
  if (lda < (N > 1 ? N : 1)) fail(EXOBLAS_INVALID_VALUE, "lda < max(1, N)");
  if (incX == 0) fail(EXOBLAS_INVALID_VALUE, "incX == 0");
  if (!A || !X) fail(EXOBLAS_INVALID_VALUE, "NULL operand");
  // rebase a negative increment as the reference wrapper does
  if (incX < 0) X = X + (1 - xlen) * long(incX);

  // scratch plan, checked against the fixed array before any work is queued
  const bool pack_x = !(incX == 1 && aligned16(X));
  const size_t xbytes = pack_x ? round256(size_t(xlen) * sizeof(float)) : 0;
  int chunks = 0;
  if (trans) {
    const long tiles = ceil_div(cols, 32 * 4);
    long want = ceil_div(long(d.sm_count) * 4, tiles);
    const long max_chunks = ceil_div(rows, 64);
    if (want > max_chunks) want = max_chunks;
    if (want < 1) want = 1;
    const long room = xbytes >= kNoAllocScratchBytes ? 0 : long((kNoAllocScratchBytes - xbytes) / (size_t(cols) * 4));
    if (room < 1)
      fail(EXOBLAS_INVALID_VALUE, "exoblas_sgemv_noalloc: problem exceeds the 4 MiB no-alloc scratch");
    // fewer chunks than exo_sgemv would use when the array is short: the
    // column sums then run in another order and can differ in the last bits
    chunks = int(want < room ? want : room);
  } else if (xbytes > kNoAllocScratchBytes) {
    fail(EXOBLAS_INVALID_VALUE, "exoblas_sgemv_noalloc: packed x exceeds the 4 MiB no-alloc scratch");
  }
  if (!on_device(A) || !on_device(X) || !on_device(Y))
    fail(EXOBLAS_INVALID_VALUE, "exoblas_sgemv_noalloc takes device pointers only");

  float *xpack = reinterpret_cast<float *>(d.scratch);
  float *partial = reinterpret_cast<float *>(d.scratch + xbytes);
  const float *xu = X;
  if (pack_x) {
    long blocks = ceil_div(xlen, kThreads);
    if (blocks > long(d.sm_count) * 4) blocks = long(d.sm_count) * 4;
    pack_kernel<float><<<int(blocks), kThreads, 0, stream>>>(xlen, X, incX, xpack);
    EXB_LAUNCH("pack kernel");
    count_launch();
    xu = xpack;
  }
  const bool vec = aligned16(A) && (long(lda) * 4) % 16 == 0;
  if (!trans) {
    const int G = cols >= 256 ? 32 : 4;
    const long rpb = (kThreads / 32) * (32 / G);
    long blocks = ceil_div(rows, rpb);
    if (blocks > long(d.sm_count) * 16) blocks = long(d.sm_count) * 16;
#define EXB_NA_ROWDOT(GG, VV) \
  rowdot_kernel<float, GG, VV, 0><<<int(blocks), kThreads, 0, stream>>>(rows, cols, alpha, A, lda, xu, beta, Y, incY, 0, false)
    if (G == 32) {
      if (vec) EXB_NA_ROWDOT(32, true);
      else EXB_NA_ROWDOT(32, false);
    } else {
      if (vec) EXB_NA_ROWDOT(4, true);
      else EXB_NA_ROWDOT(4, false);
    }
#undef EXB_NA_ROWDOT
    EXB_LAUNCH("row-dot kernel");
    count_launch();
  } else {
    const long rpc = ceil_div(rows, chunks);
    dim3 grid(unsigned(ceil_div(cols, 32 * 4)), unsigned(chunks));
    if (vec)
      colsum_kernel<float, true><<<grid, kThreads, 0, stream>>>(rows, cols, A, lda, xu, rpc, partial, 0, false);
    else
      colsum_kernel<float, false><<<grid, kThreads, 0, stream>>>(rows, cols, A, lda, xu, rpc, partial, 0, false);
    EXB_LAUNCH("column-sum kernel");
    const long blocks = finish_blocks(cols, long(d.sm_count) * 8);
    finish_kernel<float, 0><<<int(blocks), kThreads, 0, stream>>>(cols, chunks, partial, alpha, beta, Y, incY, nullptr,
                                                                 false);
    EXB_LAUNCH("partial-sum kernel");
    count_launch(2);
  }
}

}  // namespace exb

extern "C" int exoblas_sgemv_noalloc(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE TransA, const int M,
                                     const int N, const float alpha, const float *A, const int lda, const float *X,
                                     const int incX, const float beta, float *Y, const int incY, void *stream) {
  return exb::guarded("exoblas_sgemv_noalloc", [&] {
    exb::sgemv_noalloc(order, TransA, M, N, alpha, A, lda, X, incX, beta, Y, incY,
                       static_cast<cudaStream_t>(stream));
  });
}
