// exo_<p><op> level-1 entry points (C ABI).  Each one restates the special
// cases of the ExoBLAS wrapper it replaces (cited per function), stages host
// operands, launches the level-1 kernels and returns the CBLAS result.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {

template <typename T>
static inline T *rebase(T *p, long n, long inc) {
  // exo_axpy_wrapper.h:23-28 and the other wrappers: X + (1 - N) * incX
  return inc < 0 ? p + (1 - n) * inc : p;
}

static void *result_slot() { return zero_words(256) + 128; }

template <typename T>
static T fetch_result(const void *dev) {
  T v;
  EXB_CUDA(cudaMemcpyAsync(&v, dev, sizeof(T), cudaMemcpyDeviceToHost, ctx().stream));
  EXB_CUDA(cudaStreamSynchronize(ctx().stream));
  return v;
}

static bool size_ok(long n) {
  if (n < 0) fail(EXOBLAS_INVALID_VALUE, "N < 0");
  return n > 0;
}

// test/level1/asum/exo_asum_wrapper.h:5-23
template <typename T>
static T asum_entry(const char *fn, int N, const T *X, int incX) {
  T r = 0;
  guarded(fn, [&] {
    if (!size_ok(N)) return;
    if (incX < 0) return;  // exo_asum_wrapper.h:14-16
    Stager st;
    const T *dx = st.vec(X, N, incX, false);
    T *res = static_cast<T *>(result_slot());
    l1::asum<T>(N, dx, incX, res);
    r = fetch_result<T>(res);
  });
  return r;
}

// nrm2 / iamax (no reference counterpart; reference BLAS semantics).  nrm2:
// 0 for N < 1, any increment (negative walks backwards, 0 repeats x[0]);
// iamax: 0 for N < 1 or incX < 1.
template <typename T>
static T nrm2_entry(const char *fn, int N, const T *X, int incX) {
  T r = 0;
  guarded(fn, [&] {
    if (N < 1) return;
    X = rebase(X, N, incX);
    Stager st;
    const T *dx = st.vec(X, N, incX, false);
    T *res = static_cast<T *>(result_slot());
    l1::nrm2<T>(N, dx, incX, res);
    r = fetch_result<T>(res);
  });
  return r;
}
template <typename T>
static size_t iamax_entry(const char *fn, int N, const T *X, int incX) {
  size_t r = 0;
  guarded(fn, [&] {
    if (N < 1 || incX < 1) return;
    Stager st;
    const T *dx = st.vec(X, N, incX, false);
    size_t *res = static_cast<size_t *>(result_slot());
    l1::iamax<T>(N, dx, incX, res);
    r = fetch_result<size_t>(res);
  });
  return r;
}


// test/level1/axpy/exo_axpy_wrapper.h:5-34
template <typename T>
static void axpy_entry(const char *fn, int N, T alpha, const T *X, int incX, T *Y, int incY) {
  guarded(fn, [&] {
    if (alpha == T(0)) return;
    if (!size_ok(N)) return;
    if (incY == 0) fail(EXOBLAS_INVALID_VALUE, "incY == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    const T *dx = st.vec(X, N, incX, false);
    T *dy = st.vec(Y, N, incY, true);
    l1::axpy<T>(N, alpha, dx, incX, dy, incY);
    st.finish();
  });
}

// test/level1/dot/exo_dot_wrapper.h:5-27
template <typename T>
static T dot_entry(const char *fn, int N, const T *X, int incX, const T *Y, int incY) {
  T r = 0;
  guarded(fn, [&] {
    if (!size_ok(N)) return;
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    const T *dx = st.vec(X, N, incX, false);
    const T *dy = st.vec(Y, N, incY, false);
    T *res = static_cast<T *>(result_slot());
    l1::dot<T>(N, dx, incX, dy, incY, res);
    r = fetch_result<T>(res);
  });
  return r;
}

// test/level1/copy/exo_copy_wrapper.h:5-23
template <typename T>
static void copy_entry(const char *fn, int N, const T *X, int incX, T *Y, int incY) {
  guarded(fn, [&] {
    if (!size_ok(N)) return;
    if (incY == 0) fail(EXOBLAS_INVALID_VALUE, "incY == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    const T *dx = st.vec(X, N, incX, false);
    T *dy = st.vec(Y, N, incY, true);
    l1::copy<T>(N, dx, incX, dy, incY);
    st.finish();
  });
}

// test/level1/swap/exo_swap_wrapper.h:5-23
template <typename T>
static void swap_entry(const char *fn, int N, T *X, int incX, T *Y, int incY) {
  guarded(fn, [&] {
    if (!size_ok(N)) return;
    if (incX == 0 || incY == 0) fail(EXOBLAS_INVALID_VALUE, "incX == 0 or incY == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    T *dx = st.vec(X, N, incX, true);
    T *dy = st.vec(Y, N, incY, true);
    l1::swap<T>(N, dx, incX, dy, incY);
    st.finish();
  });
}

// test/level1/scal/exo_scal_wrapper.h:7-35
template <typename T>
static void scal_entry(const char *fn, int N, T alpha, T *X, int incX) {
  guarded(fn, [&] {
    if (alpha == T(1)) return;  // exo_scal_wrapper.h:10-12
    if (!size_ok(N)) return;
    if (incX < 0) return;  // exo_scal_wrapper.h:23-25
    if (incX == 0) fail(EXOBLAS_INVALID_VALUE, "incX == 0");
    Stager st;
    T *dx = st.vec(X, N, incX, true);
    l1::scal<T>(N, alpha, dx, incX);
    st.finish();
  });
}

// test/level1/rot/exo_rot_wrapper.h:5-23
template <typename T>
static void rot_entry(const char *fn, int N, T *X, int incX, T *Y, int incY, T c, T s) {
  guarded(fn, [&] {
    if (!size_ok(N)) return;
    if (incX == 0 || incY == 0) fail(EXOBLAS_INVALID_VALUE, "incX == 0 or incY == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    T *dx = st.vec(X, N, incX, true);
    T *dy = st.vec(Y, N, incY, true);
    l1::rot<T>(N, dx, incX, dy, incY, c, s);
    st.finish();
  });
}

// test/level1/rotm/exo_rotm_wrapper.h:5-44.  P is read on the host (it is a
// five-element parameter block; a device P is copied first).
template <typename T>
static void rotm_entry(const char *fn, int N, T *X, int incX, T *Y, int incY, const T *P) {
  guarded(fn, [&] {
    if (!P) fail(EXOBLAS_INVALID_VALUE, "P is NULL");
    T hp[5];
    if (is_device_pointer(P)) {
      EXB_CUDA(cudaMemcpyAsync(hp, P, sizeof hp, cudaMemcpyDeviceToHost, ctx().stream));
      EXB_CUDA(cudaStreamSynchronize(ctx().stream));
    } else {
      for (int i = 0; i < 5; ++i) hp[i] = P[i];
    }
    if (!size_ok(N)) return;
    if (!(hp[0] == T(-1) || hp[0] == T(0) || hp[0] == T(1))) return;
    if (incX == 0 || incY == 0) fail(EXOBLAS_INVALID_VALUE, "incX == 0 or incY == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    T *dx = st.vec(X, N, incX, true);
    T *dy = st.vec(Y, N, incY, true);
    l1::rotm<T>(N, dx, incX, dy, incY, hp);
    st.finish();
  });
}

// test/level1/dsdot/exo_dsdot_wrapper.h:5-25, test/level1/sdsdot/exo_sdsdot.h:5-26
static double dsdot_entry(const char *fn, int N, const float *X, int incX, const float *Y, int incY, bool sd,
                          float sb, float *sd_out) {
  double r = 0;
  guarded(fn, [&] {
    if (!size_ok(N)) {
      if (sd) *sd_out = float(0.0 + double(sb));
      return;
    }
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    const float *dx = st.vec(X, N, incX, false);
    const float *dy = st.vec(Y, N, incY, false);
    double *res = static_cast<double *>(result_slot());
    float *sres = sd ? reinterpret_cast<float *>(res + 1) : nullptr;
    l1::dsdot(N, dx, incX, dy, incY, res, sb, sres);
    if (sd)
      *sd_out = fetch_result<float>(sres);
    else
      r = fetch_result<double>(res);
  });
  return r;
}

static void require_device(const void *p, const char *what) {
  if (p && !is_device_pointer(p)) fail(EXOBLAS_INVALID_VALUE, what);
}

template <typename T>
static int asum_device(const char *fn, int N, const T *X, int incX, T *result) {
  return guarded(fn, [&] {
    require_device(X, "X must be a device pointer");
    require_device(result, "result must be a device pointer");
    if (N < 0) fail(EXOBLAS_INVALID_VALUE, "N < 0");
    if (incX < 0) N = 0;
    l1::asum<T>(N, X, incX, result);
  });
}
// device-result forms (no host synchronisation), as exoblas_?asum_device
template <typename T>
static int nrm2_device(const char *fn, int N, const T *X, int incX, T *result) {
  return guarded(fn, [&] {
    require_device(result, "result must be a device pointer");
    if (N < 1) {
      EXB_CUDA(cudaMemsetAsync(result, 0, sizeof(T), ctx().stream));
      return;
    }
    require_device(X, "X must be a device pointer");
    X = rebase(X, N, incX);
    l1::nrm2<T>(N, X, incX, result);
  });
}
template <typename T>
static int iamax_device(const char *fn, int N, const T *X, int incX, size_t *result) {
  return guarded(fn, [&] {
    require_device(result, "result must be a device pointer");
    if (N < 1 || incX < 1) {
      EXB_CUDA(cudaMemsetAsync(result, 0, sizeof(size_t), ctx().stream));
      return;
    }
    require_device(X, "X must be a device pointer");
    l1::iamax<T>(N, X, incX, result);
  });
}
template <typename T>
static int dot_device(const char *fn, int N, const T *X, int incX, const T *Y, int incY, T *result) {
  return guarded(fn, [&] {
    require_device(X, "X must be a device pointer");
    require_device(Y, "Y must be a device pointer");
    require_device(result, "result must be a device pointer");
    if (N < 0) fail(EXOBLAS_INVALID_VALUE, "N < 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    l1::dot<T>(N, X, incX, Y, incY, result);
  });
}

}  // namespace exb

using namespace exb;

extern "C" {

float exo_sasum(const int N, const float *X, const int incX) { return asum_entry<float>("exo_sasum", N, X, incX); }
float exo_snrm2(const int N, const float *X, const int incX) { return nrm2_entry<float>("exo_snrm2", N, X, incX); }
double exo_dnrm2(const int N, const double *X, const int incX) { return nrm2_entry<double>("exo_dnrm2", N, X, incX); }
size_t exo_isamax(const int N, const float *X, const int incX) {
  return iamax_entry<float>("exo_isamax", N, X, incX);
}
size_t exo_idamax(const int N, const double *X, const int incX) {
  return iamax_entry<double>("exo_idamax", N, X, incX);
}
double exo_dasum(const int N, const double *X, const int incX) { return asum_entry<double>("exo_dasum", N, X, incX); }

void exo_saxpy(const int N, const float alpha, const float *X, const int incX, float *Y, const int incY) {
  axpy_entry<float>("exo_saxpy", N, alpha, X, incX, Y, incY);
}
void exo_daxpy(const int N, const double alpha, const double *X, const int incX, double *Y, const int incY) {
  axpy_entry<double>("exo_daxpy", N, alpha, X, incX, Y, incY);
}

float exo_sdot(const int N, const float *X, const int incX, const float *Y, const int incY) {
  return dot_entry<float>("exo_sdot", N, X, incX, Y, incY);
}
double exo_ddot(const int N, const double *X, const int incX, const double *Y, const int incY) {
  return dot_entry<double>("exo_ddot", N, X, incX, Y, incY);
}

double exo_dsdot(const int N, const float *X, const int incX, const float *Y, const int incY) {
  return dsdot_entry("exo_dsdot", N, X, incX, Y, incY, false, 0.f, nullptr);
}
float exo_sdsdot(const int N, const float alpha, const float *X, const int incX, const float *Y, const int incY) {
  float r = 0.f;
  dsdot_entry("exo_sdsdot", N, X, incX, Y, incY, true, alpha, &r);
  return r;
}

void exo_scopy(const int N, const float *X, const int incX, float *Y, const int incY) {
  copy_entry<float>("exo_scopy", N, X, incX, Y, incY);
}
void exo_dcopy(const int N, const double *X, const int incX, double *Y, const int incY) {
  copy_entry<double>("exo_dcopy", N, X, incX, Y, incY);
}
void exo_sswap(const int N, float *X, const int incX, float *Y, const int incY) {
  swap_entry<float>("exo_sswap", N, X, incX, Y, incY);
}
void exo_dswap(const int N, double *X, const int incX, double *Y, const int incY) {
  swap_entry<double>("exo_dswap", N, X, incX, Y, incY);
}
void exo_sscal(const int N, const float alpha, float *X, const int incX) {
  scal_entry<float>("exo_sscal", N, alpha, X, incX);
}
void exo_dscal(const int N, const double alpha, double *X, const int incX) {
  scal_entry<double>("exo_dscal", N, alpha, X, incX);
}
void exo_srot(const int N, float *X, const int incX, float *Y, const int incY, const float c, const float s) {
  rot_entry<float>("exo_srot", N, X, incX, Y, incY, c, s);
}
void exo_drot(const int N, double *X, const int incX, double *Y, const int incY, const double c, const double s) {
  rot_entry<double>("exo_drot", N, X, incX, Y, incY, c, s);
}
void exo_srotm(const int N, float *X, const int incX, float *Y, const int incY, const float *P) {
  rotm_entry<float>("exo_srotm", N, X, incX, Y, incY, P);
}
void exo_drotm(const int N, double *X, const int incX, double *Y, const int incY, const double *P) {
  rotm_entry<double>("exo_drotm", N, X, incX, Y, incY, P);
}

int exoblas_snrm2_device(const int N, const float *X, const int incX, float *result) {
  return nrm2_device<float>("exoblas_snrm2_device", N, X, incX, result);
}
int exoblas_dnrm2_device(const int N, const double *X, const int incX, double *result) {
  return nrm2_device<double>("exoblas_dnrm2_device", N, X, incX, result);
}
int exoblas_isamax_device(const int N, const float *X, const int incX, size_t *result) {
  return iamax_device<float>("exoblas_isamax_device", N, X, incX, result);
}
int exoblas_idamax_device(const int N, const double *X, const int incX, size_t *result) {
  return iamax_device<double>("exoblas_idamax_device", N, X, incX, result);
}
int exoblas_sasum_device(const int N, const float *X, const int incX, float *result) {
  return asum_device<float>("exoblas_sasum_device", N, X, incX, result);
}
int exoblas_dasum_device(const int N, const double *X, const int incX, double *result) {
  return asum_device<double>("exoblas_dasum_device", N, X, incX, result);
}
int exoblas_sdot_device(const int N, const float *X, const int incX, const float *Y, const int incY, float *result) {
  return dot_device<float>("exoblas_sdot_device", N, X, incX, Y, incY, result);
}
int exoblas_ddot_device(const int N, const double *X, const int incX, const double *Y, const int incY,
                        double *result) {
  return dot_device<double>("exoblas_ddot_device", N, X, incX, Y, incY, result);
}
int exoblas_dsdot_device(const int N, const float *X, const int incX, const float *Y, const int incY,
                         double *result) {
  return guarded("exoblas_dsdot_device", [&] {
    require_device(X, "X must be a device pointer");
    require_device(Y, "Y must be a device pointer");
    require_device(result, "result must be a device pointer");
    if (N < 0) fail(EXOBLAS_INVALID_VALUE, "N < 0");
    const float *x = rebase(X, N, incX), *y = rebase(Y, N, incY);
    l1::dsdot(N, x, incX, y, incY, result, 0.f, nullptr);
  });
}

}  // extern "C"
