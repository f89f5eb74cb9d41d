// Per-thread execution state, workspace arenas, status reporting and the
// host-operand staging used by every exo_* entry point.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "common.cuh"
#include "runtime.h"

namespace exb {

static std::atomic<unsigned long long> g_launches{0};
static std::atomic<unsigned long long> g_h2d{0}, g_d2h{0};
void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static thread_local int tl_status = EXOBLAS_SUCCESS;
static exoblas_error_handler g_handler = nullptr;

void fail(int status, const char *what) { throw Error{status, what}; }

void check_cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return;
  static thread_local char buf[512];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorMemoryAllocation) throw Error{EXOBLAS_ALLOC_FAILED, buf};
  throw Error{EXOBLAS_CUDA_ERROR, buf};
}

void *Arena::get(size_t need) {
  if (need == 0) need = 256;
  if (need <= bytes) return ptr;
  if (ptr) {
    // the previous buffer may still be read by queued work of this thread
    cudaStreamSynchronize(ctx().stream);
    cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
  size_t want = need + need / 4;
  want = (want + 0xFFFFF) & ~size_t(0xFFFFF);  // whole MiB
  cudaError_t e = cudaMalloc(&ptr, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaMalloc(&ptr, need);
    want = need;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    ptr = nullptr;
    fail(EXOBLAS_ALLOC_FAILED, "device workspace allocation failed");
  }
  bytes = want;
  return ptr;
}

void Arena::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

Context::~Context() {
  // Runs at thread exit; the CUDA runtime may already be shutting down at
  // process exit, so errors are ignored.
  scratch.release();
  counters.release();
  for (auto &s : staging) s.release();
  if (own_stream && stream) cudaStreamDestroy(stream);
  if (side) cudaStreamDestroy(side);
  if (fork) cudaEventDestroy(fork);
  if (join) cudaEventDestroy(join);
  cudaGetLastError();
}

static int initial_precision() {
  const char *e = getenv("EXOBLAS_PRECISION_MODE");
  if (!e) return EXOBLAS_PRECISION_NATIVE;
  if (!strcmp(e, "split_bf16")) return EXOBLAS_PRECISION_SPLIT_BF16;
  if (!strcmp(e, "ozaki")) return EXOBLAS_PRECISION_OZAKI;
  return EXOBLAS_PRECISION_NATIVE;
}

static int initial_column_major() {
  const char *e = getenv("EXOBLAS_COLUMN_MAJOR");
  return e && (!strcmp(e, "1") || !strcmp(e, "on")) ? 1 : 0;
}
static thread_local int tl_column_major = initial_column_major();

constexpr int kMaxDevices = 64;
static thread_local Context *tl_ctx[kMaxDevices] = {};
struct CtxOwner {
  ~CtxOwner() {
    for (auto &c : tl_ctx) {
      delete c;
      c = nullptr;
    }
  }
};
static thread_local CtxOwner tl_owner;

bool column_major_enabled() { return tl_column_major != 0; }

Context &ctx() {
  int dev = 0;
  EXB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) fail(EXOBLAS_NOT_SUPPORTED, "device index out of range");
  Context *&c = tl_ctx[dev];
  if (!c) {
    (void)&tl_owner;
    Context *n = new Context();
    n->device = dev;
    n->precision = initial_precision();
    cudaDeviceProp prop;
    EXB_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (prop.major < 10) {
      delete n;
      fail(EXOBLAS_NOT_SUPPORTED, "libexoblas_gb300 requires a Blackwell (sm_103) device");
    }
    n->sm_count = prop.multiProcessorCount;
    int pa = 0, pt = 0;
    if (cudaDeviceGetAttribute(&pa, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) {
      cudaGetLastError();
      pa = pt = 0;
    }
    n->pageable_direct = pa != 0 && pt != 0;
    EXB_CUDA(cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking));
    n->own_stream = true;
    c = n;
  }
  return *c;
}

void *scratch(size_t bytes) { return ctx().scratch.get((bytes + 255) & ~size_t(255)); }

unsigned int *zero_words(int n) {
  Context &c = ctx();
  const size_t need = size_t(n) * 4;
  if (c.counters.bytes < need) {
    c.counters.get(need < 4096 ? 4096 : need);
    EXB_CUDA(cudaMemsetAsync(c.counters.ptr, 0, c.counters.bytes, c.stream));
  }
  return static_cast<unsigned int *>(c.counters.ptr);
}

// ---------------------------------------------------------------- staging --

bool is_device_pointer(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Copies between pageable host memory and the staging buffers.  Where the
// device reads pageable memory through the host page tables (Grace + ATS),
// a grid-stride copy kernel moves the bytes over the C2C link with no host
// work: cudaMemcpy's pageable path needs the host side, and its rate varied
// from 5 to 193 GB/s across otherwise identical boxes (this kernel: 208 GB/s
// host to device, 187 GB/s device to host; pinned DMA copies 210 GB/s).
// Pinned memory keeps cudaMemcpy.
template <typename V>
__global__ void __launch_bounds__(512) host_copy_kernel(const V *__restrict__ s, V *__restrict__ d, size_t n) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    d[i] = s[i];
}

static bool pageable(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeUnregistered;
}

// contiguous copy of `bytes`; `host` is the host side's pointer
static void host_copy(Context &c, void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, const void *host) {
  if (!c.pageable_direct || !pageable(host)) {
    EXB_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, c.stream));
    return;
  }
  const uintptr_t a = reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst) | uintptr_t(bytes);
  const size_t g = (a & 15) == 0 ? 16 : (a & 7) == 0 ? 8 : (a & 3) == 0 ? 4 : 1;
  const size_t n = bytes / g;
  long blocks = long((n + 511) / 512);
  if (blocks > 4L * c.sm_count) blocks = 4L * c.sm_count;
  if (blocks < 1) blocks = 1;
  switch (g) {
    case 16:
      host_copy_kernel<<<unsigned(blocks), 512, 0, c.stream>>>(static_cast<const uint4 *>(src), static_cast<uint4 *>(dst), n);
      break;
    case 8:
      host_copy_kernel<<<unsigned(blocks), 512, 0, c.stream>>>(static_cast<const uint2 *>(src), static_cast<uint2 *>(dst), n);
      break;
    case 4:
      host_copy_kernel<<<unsigned(blocks), 512, 0, c.stream>>>(static_cast<const unsigned *>(src), static_cast<unsigned *>(dst), n);
      break;
    default:
      host_copy_kernel<<<unsigned(blocks), 512, 0, c.stream>>>(static_cast<const unsigned char *>(src), static_cast<unsigned char *>(dst), n);
  }
  EXB_LAUNCH("host copy kernel");
  count_launch();
}

Stager::Stager() : c(ctx()) {}

void *Stager::stage(const void *p, size_t elem, long count, long inc, bool out) {
  // Span of a strided vector whose element 0 is at p and element i at p + i*inc
  if (count <= 0 || !p) return const_cast<void *>(p);
  if (is_device_pointer(p)) return const_cast<void *>(p);
  const long lo = inc < 0 ? (count - 1) * inc : 0;
  const long hi = inc < 0 ? 0 : (count - 1) * inc;
  const size_t bytes = size_t(hi - lo + 1) * elem;
  const char *base = static_cast<const char *>(p) + lo * long(elem);
  if (nslots >= kSlots) fail(EXOBLAS_INVALID_VALUE, "too many host operands");
  char *d = static_cast<char *>(c.staging[nslots].get(bytes));
  host_copy(c, d, base, bytes, cudaMemcpyHostToDevice, base);
  Slot &s = slots[nslots++];
  s = Slot{const_cast<char *>(base), d, bytes, 0, 0, 0, out};
  any_host = true;
  h2d += bytes;
  g_h2d.fetch_add(bytes, std::memory_order_relaxed);
  return d - lo * long(elem);
}

void *Stager::stage_matrix(const void *p, size_t elem, long rows, long cols, long ld, bool out) {
  if (rows <= 0 || cols <= 0 || !p) return const_cast<void *>(p);
  if (is_device_pointer(p)) return const_cast<void *>(p);
  const size_t bytes = size_t((rows - 1) * ld + cols) * elem;
  if (nslots >= kSlots) fail(EXOBLAS_INVALID_VALUE, "too many host operands");
  char *d = static_cast<char *>(c.staging[nslots].get(bytes));
  const size_t pitch = size_t(ld) * elem, width = size_t(cols) * elem;
  if (ld == cols)
    host_copy(c, d, p, bytes, cudaMemcpyHostToDevice, p);
  else
    EXB_CUDA(cudaMemcpy2DAsync(d, pitch, p, pitch, width, rows, cudaMemcpyHostToDevice, c.stream));
  Slot &s = slots[nslots++];
  s = Slot{const_cast<void *>(p), d, bytes, pitch, width, size_t(rows), out};
  any_host = true;
  h2d += size_t(rows) * width;
  g_h2d.fetch_add(size_t(rows) * width, std::memory_order_relaxed);
  return d;
}

void Stager::finish() {
  for (int i = 0; i < nslots; ++i) {
    Slot &s = slots[i];
    if (!s.out) continue;
    g_d2h.fetch_add(s.rows ? s.rows * s.width : s.bytes, std::memory_order_relaxed);
    if (s.rows) {
      // matrices: copy back only the rows' used columns so padding between
      // rows (ld > cols) is never written
      if (s.pitch == s.width)
        host_copy(c, s.host, s.dev, s.bytes, cudaMemcpyDeviceToHost, s.host);
      else
        EXB_CUDA(cudaMemcpy2DAsync(s.host, s.pitch, s.dev, s.pitch, s.width, s.rows, cudaMemcpyDeviceToHost,
                                   c.stream));
    } else {
      host_copy(c, s.host, s.dev, s.bytes, cudaMemcpyDeviceToHost, s.host);
    }
  }
  if (any_host || c.blocking) {
    EXB_CUDA(cudaStreamSynchronize(c.stream));
    check_device_status();
  }
}

// Device status word written by kernels with bounded waits.
int *device_status_word() { return reinterpret_cast<int *>(zero_words(64) + 32); }

void set_status(int s) { tl_status = s; }

// Reads (after the caller synchronised the stream) and clears the device
// status word; a nonzero value means a bounded wait ran out.
void check_device_status() {
  Context &c = ctx();
  if (!c.status_pending) return;
  c.status_pending = false;
  int st = 0;
  int *w = device_status_word();
  EXB_CUDA(cudaMemcpyAsync(&st, w, 4, cudaMemcpyDeviceToHost, c.stream));
  EXB_CUDA(cudaStreamSynchronize(c.stream));
  if (st) {
    EXB_CUDA(cudaMemsetAsync(w, 0, 4, c.stream));
    EXB_CUDA(cudaStreamSynchronize(c.stream));
    fail(EXOBLAS_TIMEOUT, "a kernel's bounded wait ran out");
  }
}

void report(int status, const char *fn, const char *msg) {
  tl_status = status;
  if (g_handler) g_handler(status, fn, msg);
}

}  // namespace exb

using namespace exb;

// A wait on a device flag that nothing sets, bounded by `limit_ns` of the
// global timer; on expiry it records the timeout in the status word, as the
// solvers' bounded waits do, and returns.
__global__ void expiring_wait_kernel(const int *flag, unsigned long long limit_ns, int *status) {
  if (threadIdx.x != 0) return;
  unsigned long long t0, t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
  for (;;) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
    if (v != 0) return;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    if (t - t0 > limit_ns) {
      atomicExch(status, 1);
      return;
    }
    __nanosleep(1000);
  }
}

extern "C" {

int exoblas_get_status(void) { return tl_status; }

const char *exoblas_status_string(int s) {
  switch (s) {
    case EXOBLAS_SUCCESS: return "success";
    case EXOBLAS_UNSUPPORTED_ORDER: return "Order must be CblasRowMajor";
    case EXOBLAS_INVALID_VALUE: return "invalid argument";
    case EXOBLAS_CUDA_ERROR: return "CUDA error";
    case EXOBLAS_ALLOC_FAILED: return "device allocation failed";
    case EXOBLAS_TIMEOUT: return "kernel wait timed out";
    case EXOBLAS_NOT_SUPPORTED: return "not supported on this device";
    default: return "unknown status";
  }
}

void exoblas_set_error_handler(exoblas_error_handler h) { g_handler = h; }

int exoblas_set_stream(void *stream) {
  return guarded("exoblas_set_stream", [&] {
    Context &c = ctx();
    EXB_CUDA(cudaStreamSynchronize(c.stream));
    if (stream) {
      if (c.own_stream) EXB_CUDA(cudaStreamDestroy(c.stream));
      c.stream = static_cast<cudaStream_t>(stream);
      c.own_stream = false;
    } else if (!c.own_stream) {
      EXB_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
      c.own_stream = true;
    }
  });
}

void *exoblas_get_stream(void) {
  void *s = nullptr;
  guarded("exoblas_get_stream", [&] { s = ctx().stream; });
  return s;
}

int exoblas_set_blocking(int b) {
  return guarded("exoblas_set_blocking", [&] { ctx().blocking = b != 0; });
}

int exoblas_synchronize(void) {
  return guarded("exoblas_synchronize", [&] {
    EXB_CUDA(cudaStreamSynchronize(ctx().stream));
    check_device_status();
  });
}

int exoblas_set_precision(int mode) {
  return guarded("exoblas_set_precision", [&] {
    if (mode < EXOBLAS_PRECISION_NATIVE || mode > EXOBLAS_PRECISION_OZAKI)
      fail(EXOBLAS_INVALID_VALUE, "unknown precision mode");
    ctx().precision = mode;
  });
}

int exoblas_set_column_major(int enable) {
  tl_column_major = enable ? 1 : 0;
  return EXOBLAS_SUCCESS;
}

int exoblas_get_column_major(void) { return tl_column_major; }

int exoblas_get_precision(void) {
  int p = EXOBLAS_PRECISION_NATIVE;
  guarded("exoblas_get_precision", [&] { p = ctx().precision; });
  return p;
}

int exoblas_selftest_wait_timeout(double seconds) {
  return guarded("exoblas_selftest_wait_timeout", [&] {
    if (!(seconds > 0.0 && seconds <= 1.0)) fail(EXOBLAS_INVALID_VALUE, "seconds must lie in (0, 1]");
    Context &c = ctx();
    int *flag = static_cast<int *>(scratch(256));
    EXB_CUDA(cudaMemsetAsync(flag, 0, 4, c.stream));
    expiring_wait_kernel<<<1, 32, 0, c.stream>>>(flag, static_cast<unsigned long long>(seconds * 1e9),
                                                 device_status_word());
    EXB_LAUNCH("expiring-wait kernel");
    count_launch();
    c.status_pending = true;
    EXB_CUDA(cudaStreamSynchronize(c.stream));
    check_device_status();  // the recorded expiry surfaces as EXOBLAS_TIMEOUT
  });
}

unsigned long long exoblas_kernel_launches(void) { return g_launches.load(); }

void exoblas_staged_bytes(unsigned long long *h2d, unsigned long long *d2h) {
  if (h2d) *h2d = g_h2d.load();
  if (d2h) *d2h = g_d2h.load();
}

}  // extern "C"

namespace exb {

int resident_per_sm(const void *kernel, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, int> cache;
  const int dev = ctx().device;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({dev, kernel});
    if (it != cache.end()) return it->second;
  }
  int per_sm = 0;
  EXB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
  if (per_sm < 1) per_sm = 1;
  std::lock_guard<std::mutex> lk(mu);
  cache[{dev, kernel}] = per_sm;
  return per_sm;
}

long balanced_grid(long want, const void *kernel, int threads, size_t smem) {
  if (want < 1) return 1;
  const long wave = long(ctx().sm_count) * resident_per_sm(kernel, threads, smem);
  const long waves = ceil_div(want, wave);
  return ceil_div(want, waves);
}

}  // namespace exb
