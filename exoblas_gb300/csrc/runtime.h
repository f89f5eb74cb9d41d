// Host-side runtime interface shared by the entry points and the launchers.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "common.cuh"

namespace exb {

void count_launch(unsigned n = 1);
// column-major calls accepted on this thread (exoblas_set_column_major)
bool column_major_enabled();
// CTAs of `kernel` (threads per CTA, dynamic shared memory) resident at once
// on one SM of the current device; cached per device and kernel.
int resident_per_sm(const void *kernel, int threads, size_t smem = 0);
// a grid of at most `want` CTAs that runs in whole waves of equal work:
// want is split into the fewest waves of the device's resident CTAs and the
// grid is the per-wave share, so every CTA of a grid-stride loop gets the
// same number of items
long balanced_grid(long want, const void *kernel, int threads, size_t smem = 0);
bool is_device_pointer(const void *p);
void set_status(int s);
void report(int status, const char *fn, const char *msg);
// Device word (in the zeroed counter region) where kernels with bounded
// waits record a timeout; the host reads and clears it after the call.
int *device_status_word();
// After a stream synchronisation: raises EXOBLAS_TIMEOUT if a kernel queued
// since the last check recorded an expired wait (see Context::status_pending).
void check_device_status();

// Runs `body`, converting library errors into the thread's status.  Returns
// the status (0 on success).
template <typename F>
int guarded(const char *fn, F &&body) {
  try {
    set_status(EXOBLAS_SUCCESS);
    body();
    return EXOBLAS_SUCCESS;
  } catch (const Error &e) {
    report(e.status, fn, e.what);
    return e.status;
  } catch (...) {
    report(EXOBLAS_CUDA_ERROR, fn, "unexpected exception");
    return EXOBLAS_CUDA_ERROR;
  }
}

// Host-operand staging for one call: each host pointer is copied into a
// device slot; device pointers pass through unchanged.  finish() copies the
// outputs back and waits when a host operand was involved or the thread is
// in blocking mode.
class Stager {
 public:
  Stager();
  // Strided vector: element 0 at p, element i at p + i*inc (inc may be < 0).
  template <typename T>
  T *vec(const T *p, long n, long inc, bool out) {
    return static_cast<T *>(stage(p, sizeof(T), n, inc, out));
  }
  // Row-major rows x cols matrix with leading dimension ld.
  template <typename T>
  T *mat(const T *p, long rows, long cols, long ld, bool out) {
    return static_cast<T *>(stage_matrix(p, sizeof(T), rows, cols, ld, out));
  }
  void finish();
  bool host_involved() const { return any_host; }
  Context &c;

 private:
  void *stage(const void *p, size_t elem, long count, long inc, bool out);
  void *stage_matrix(const void *p, size_t elem, long rows, long cols, long ld, bool out);
  struct Slot {
    void *host;
    char *dev;
    size_t bytes, pitch, width, rows;
    bool out;
  };
  static constexpr int kSlots = 6;
  Slot slots[kSlots];
  int nslots = 0;
  bool any_host = false;
  size_t h2d = 0;
};

}  // namespace exb
