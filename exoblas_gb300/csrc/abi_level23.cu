// exo_<p><op> level-2 and level-3 entry points (C ABI).  Flag handling is
// the reference's: each proc tests one flag value and takes the other branch
// for anything else (e.g. gemv.py:15 tests TransA == NoTrans, trmv.py:23
// tests Diag == Unit, trsv.py:29 tests Diag == NonUnit), so the same
// permissive mapping is used here.  Arguments the reference never checks
// but that would make a GPU kernel read or write out of bounds (negative
// sizes, a leading dimension smaller than the row length, a zero output
// stride) are rejected with EXOBLAS_INVALID_VALUE and leave outputs untouched.
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"
#include "runtime.h"

namespace exb {

template <typename T>
static inline T *rebase(T *p, long n, long inc) {
  return inc < 0 ? p + (1 - n) * inc : p;
}

static void row_major(int order) {
  if (order != kRowMajor) fail(EXOBLAS_UNSUPPORTED_ORDER, "Order must be CblasRowMajor");
}
static void nonneg(long v, const char *what) {
  if (v < 0) fail(EXOBLAS_INVALID_VALUE, what);
}
static void ld_ok(long ld, long cols, const char *what) {
  if (ld < (cols > 1 ? cols : 1)) fail(EXOBLAS_INVALID_VALUE, what);
}
static void inc_ok(long inc, const char *what) {
  if (inc == 0) fail(EXOBLAS_INVALID_VALUE, what);
}

// Level-3 dispatch on the thread's precision mode.
static bool split_mode() { return ctx().precision == EXOBLAS_PRECISION_SPLIT_BF16; }

static void gemm_dispatch(bool ta, bool tb, long m, long n, long k, float alpha, const float *A, long lda,
                          const float *B, long ldb, float beta, float *C, long ldc) {
  if (split_mode() && k > 0)
    l3::gemm_split_bf16(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else
    l3::gemm_simt<float>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
static void gemm_dispatch(bool ta, bool tb, long m, long n, long k, double alpha, const double *A, long lda,
                          const double *B, long ldb, double beta, double *C, long ldc) {
  if (ctx().precision == EXOBLAS_PRECISION_OZAKI && k > 0 &&
      l3::dgemm_ozaki(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc))
    return;
  l3::gemm_simt<double>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
static void symm_dispatch(bool left, bool upper, long m, long n, float alpha, const float *A, long lda, const float *B,
                          long ldb, float beta, float *C, long ldc) {
  if (split_mode())
    l3::symm_split_bf16(left, upper, m, n, alpha, A, lda, B, ldb, beta, C, ldc);
  else
    l3::symm_simt<float>(left, upper, m, n, alpha, A, lda, B, ldb, beta, C, ldc);
}
static void symm_dispatch(bool left, bool upper, long m, long n, double alpha, const double *A, long lda,
                          const double *B, long ldb, double beta, double *C, long ldc) {
  if (ctx().precision == EXOBLAS_PRECISION_OZAKI && l3::dsymm_ozaki(left, upper, m, n, alpha, A, lda, B, ldb, beta, C, ldc))
    return;
  l3::symm_simt<double>(left, upper, m, n, alpha, A, lda, B, ldb, beta, C, ldc);
}
static void syrk_dispatch(bool upper, bool trans, long n, long k, float alpha, const float *A, long lda, float beta,
                          float *C, long ldc) {
  if (split_mode() && k > 0)
    l3::syrk_split_bf16(upper, trans, n, k, alpha, A, lda, beta, C, ldc);
  else
    l3::syrk_simt<float>(upper, trans, n, k, alpha, A, lda, beta, C, ldc);
}
static void syrk_dispatch(bool upper, bool trans, long n, long k, double alpha, const double *A, long lda, double beta,
                          double *C, long ldc) {
  if (ctx().precision == EXOBLAS_PRECISION_OZAKI && k > 0 &&
      l3::dsyrk_ozaki(upper, trans, n, k, alpha, A, lda, beta, C, ldc))
    return;
  l3::syrk_simt<double>(upper, trans, n, k, alpha, A, lda, beta, C, ldc);
}
static void syr2k_dispatch(bool upper, bool trans, long n, long k, float alpha, const float *A, long lda,
                           const float *B, long ldb, float beta, float *C, long ldc) {
  if (split_mode() && k > 0)
    l3::syr2k_split_bf16(upper, trans, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  else
    l3::syr2k_simt<float>(upper, trans, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}
static void syr2k_dispatch(bool upper, bool trans, long n, long k, double alpha, const double *A, long lda,
                           const double *B, long ldb, double beta, double *C, long ldc) {
  if (ctx().precision == EXOBLAS_PRECISION_OZAKI && k > 0 &&
      l3::dsyr2k_ozaki(upper, trans, n, k, alpha, A, lda, B, ldb, beta, C, ldc))
    return;
  l3::syr2k_simt<double>(upper, trans, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
}

// ------------------------------------------------------------------ level 2

// test/level2/gemv/exo_gemv_wrapper.h:7-39
template <typename T>
static void gemv_entry(const char *fn, int order, int TransA, int M, int N, T alpha, const T *A, int lda, const T *X,
                       int incX, T beta, T *Y, int incY) {
  guarded(fn, [&] {
    row_major(order);
    nonneg(M, "M < 0");
    nonneg(N, "N < 0");
    const bool trans = TransA != kNoTrans;
    const long ylen = trans ? N : M, xlen = trans ? M : N;
    if (ylen == 0) return;
    if (M > 0 && N > 0) ld_ok(lda, N, "lda < max(1, N)");
    inc_ok(incY, "incY == 0");
    if (xlen > 0) inc_ok(incX, "incX == 0");
    X = rebase(X, xlen, incX);
    Y = rebase(Y, ylen, incY);
    Stager st;
    const T *dA = st.mat(A, M, N, lda, false);
    const T *dx = st.vec(X, xlen, incX, false);
    T *dy = st.vec(Y, ylen, incY, true);
    l2::gemv<T>(trans, M, N, alpha, dA, lda, dx, incX, beta, dy, incY);
    st.finish();
  });
}

// test/level2/ger/exo_ger_wrapper.h:7-34 (Order not checked)
template <typename T>
static void ger_entry(const char *fn, int M, int N, T alpha, const T *X, int incX, const T *Y, int incY, T *A,
                      int lda) {
  guarded(fn, [&] {
    if (alpha == T(0)) return;
    nonneg(M, "M < 0");
    nonneg(N, "N < 0");
    if (M == 0 || N == 0) return;
    ld_ok(lda, N, "lda < max(1, N)");
    inc_ok(incX, "incX == 0");
    inc_ok(incY, "incY == 0");
    X = rebase(X, M, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    const T *dx = st.vec(X, M, incX, false);
    const T *dy = st.vec(Y, N, incY, false);
    T *dA = st.mat(A, M, N, lda, true);
    l2::ger<T>(M, N, alpha, dx, incX, dy, incY, dA, lda);
    st.finish();
  });
}

// test/level2/symv/exo_symv_wrapper.h:7-34
template <typename T>
static void symv_entry(const char *fn, int order, int Uplo, int N, T alpha, const T *A, int lda, const T *X, int incX,
                       T beta, T *Y, int incY) {
  guarded(fn, [&] {
    row_major(order);
    nonneg(N, "N < 0");
    if (N == 0) return;
    ld_ok(lda, N, "lda < max(1, N)");
    inc_ok(incX, "incX == 0");
    inc_ok(incY, "incY == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    const T *dA = st.mat(A, N, N, lda, false);
    const T *dx = st.vec(X, N, incX, false);
    T *dy = st.vec(Y, N, incY, true);
    l2::symv<T>(Uplo == kUpper, N, alpha, dA, lda, dx, incX, beta, dy, incY);
    st.finish();
  });
}

// test/level2/syr/exo_syr_wrapper.h:5-32
template <typename T>
static void syr_entry(const char *fn, int order, int Uplo, int N, T alpha, const T *X, int incX, T *A, int lda) {
  guarded(fn, [&] {
    row_major(order);
    if (alpha == T(0)) return;
    nonneg(N, "N < 0");
    if (N == 0) return;
    ld_ok(lda, N, "lda < max(1, N)");
    inc_ok(incX, "incX == 0");
    X = rebase(X, N, incX);
    Stager st;
    const T *dx = st.vec(X, N, incX, false);
    T *dA = st.mat(A, N, N, lda, true);
    l2::syr<T>(Uplo == kUpper, N, alpha, dx, incX, dA, lda);
    st.finish();
  });
}

// test/level2/syr2/exo_syr2_wrapper.h:5-36 (Order not checked)
template <typename T>
static void syr2_entry(const char *fn, int Uplo, int N, T alpha, const T *X, int incX, const T *Y, int incY, T *A,
                       int lda) {
  guarded(fn, [&] {
    if (alpha == T(0)) return;
    nonneg(N, "N < 0");
    if (N == 0) return;
    ld_ok(lda, N, "lda < max(1, N)");
    inc_ok(incX, "incX == 0");
    inc_ok(incY, "incY == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    const T *dx = st.vec(X, N, incX, false);
    const T *dy = st.vec(Y, N, incY, false);
    T *dA = st.mat(A, N, N, lda, true);
    l2::syr2<T>(Uplo == kUpper, N, alpha, dx, incX, dy, incY, dA, lda);
    st.finish();
  });
}

// test/level2/trmv/exo_trmv_wrapper.h:7-29 (unit diagonal iff Diag == Unit, trmv.py:23)
// test/level2/trsv/exo_trsv_wrapper.h:7-29 (divides iff Diag == NonUnit, trsv.py:29)
template <typename T, bool SOLVE>
static void tr_entry(const char *fn, int order, int Uplo, int TransA, int Diag, int N, const T *A, int lda, T *X,
                     int incX) {
  guarded(fn, [&] {
    row_major(order);
    nonneg(N, "N < 0");
    if (N == 0) return;
    ld_ok(lda, N, "lda < max(1, N)");
    inc_ok(incX, "incX == 0");
    X = rebase(X, N, incX);
    Stager st;
    const T *dA = st.mat(A, N, N, lda, false);
    T *dx = st.vec(X, N, incX, true);
    const bool upper = Uplo == kUpper, trans = TransA != kNoTrans;
    if (SOLVE)
      l2::trsv<T>(upper, trans, Diag != kNonUnit, N, dA, lda, dx, incX);
    else
      l2::trmv<T>(upper, trans, Diag == kUnit, N, dA, lda, dx, incX);
    st.finish();
  });
}

// ------------------------------------------------------------------ level 3

// test/level3/gemm/exo_gemm_wrapper.h:9-28
template <typename T>
static void gemm_entry(const char *fn, int Order, int TransA, int TransB, int M, int N, int K, T alpha, const T *A,
                       int lda, const T *B, int ldb, T beta, T *C, int ldc) {
  guarded(fn, [&] {
    row_major(Order);
    nonneg(M, "M < 0");
    nonneg(N, "N < 0");
    nonneg(K, "K < 0");
    if (M == 0 || N == 0) return;
    const bool ta = TransA != kNoTrans, tb = TransB != kNoTrans;
    const long ar = ta ? K : M, ac = ta ? M : K, br = tb ? N : K, bc = tb ? K : N;
    if (K > 0) {
      ld_ok(lda, ac, "lda too small");
      ld_ok(ldb, bc, "ldb too small");
    }
    ld_ok(ldc, N, "ldc < max(1, N)");
    Stager st;
    const T *dA = K > 0 ? st.mat(A, ar, ac, lda, false) : A;
    const T *dB = K > 0 ? st.mat(B, br, bc, ldb, false) : B;
    T *dC = st.mat(C, M, N, ldc, true);
    gemm_dispatch(ta, tb, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc);
    st.finish();
  });
}

// test/level3/symm/exo_symm_wrapper.h:9-27
template <typename T>
static void symm_entry(const char *fn, int Order, int Side, int Uplo, int M, int N, T alpha, const T *A, int lda,
                       const T *B, int ldb, T beta, T *C, int ldc) {
  guarded(fn, [&] {
    row_major(Order);
    nonneg(M, "M < 0");
    nonneg(N, "N < 0");
    if (M == 0 || N == 0) return;
    const bool left = Side == kLeft;
    const long ka = left ? M : N;
    ld_ok(lda, ka, "lda too small");
    ld_ok(ldb, N, "ldb < max(1, N)");
    ld_ok(ldc, N, "ldc < max(1, N)");
    Stager st;
    const T *dA = st.mat(A, ka, ka, lda, false);
    const T *dB = st.mat(B, M, N, ldb, false);
    T *dC = st.mat(C, M, N, ldc, true);
    symm_dispatch(left, Uplo == kUpper, M, N, alpha, dA, lda, dB, ldb, beta, dC, ldc);
    st.finish();
  });
}

// test/level3/syrk/exo_syrk_wrapper.h:9-28
template <typename T>
static void syrk_entry(const char *fn, int Order, int Uplo, int Trans, int N, int K, T alpha, const T *A, int lda,
                       T beta, T *C, int ldc) {
  guarded(fn, [&] {
    row_major(Order);
    nonneg(N, "N < 0");
    nonneg(K, "K < 0");
    if (N == 0) return;
    const bool trans = Trans != kNoTrans;
    const long ar = trans ? K : N, ac = trans ? N : K;
    if (K > 0) ld_ok(lda, ac, "lda too small");
    ld_ok(ldc, N, "ldc < max(1, N)");
    Stager st;
    const T *dA = K > 0 ? st.mat(A, ar, ac, lda, false) : A;
    T *dC = st.mat(C, N, N, ldc, true);
    syrk_dispatch(Uplo == kUpper, trans, N, K, alpha, dA, lda, beta, dC, ldc);
    st.finish();
  });
}

// test/level2/sgbmv/exo_sgbmv.h:5-23 (no Order or Trans argument: row-major
// NoTrans).  The reference passes negative increments through unrebased,
// which reads before X; here they follow the CBLAS convention (rebased).
template <typename T>
static void gbmv_entry(const char *fn, int M, int N, int KL, int KU, T alpha, const T *A, int lda, const T *X,
                       int incX, T beta, T *Y, int incY) {
  guarded(fn, [&] {
    nonneg(M, "M < 0");
    nonneg(N, "N < 0");
    nonneg(KL, "KL < 0");
    nonneg(KU, "KU < 0");
    if (M == 0) return;
    const long width = long(KL) + KU + 1;
    ld_ok(lda, width, "lda < KL + KU + 1");
    inc_ok(incY, "incY == 0");
    if (N > 0) inc_ok(incX, "incX == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, M, incY);
    Stager st;
    const T *dA = st.mat(A, M, width, lda, false);
    const T *dx = st.vec(X, N, incX, false);
    T *dy = st.vec(Y, M, incY, true);
    l2::gbmv<T>(M, N, KL, KU, alpha, dA, lda, dx, incX, beta, dy, incY);
    st.finish();
  });
}

// test/level2/ssbmv/exo_ssbmv.h:7-52: y = beta y (when beta != 1) then
// y += alpha A x; Uplo other than Upper reads the lower band.
template <typename T>
static void sbmv_entry(const char *fn, int order, int Uplo, int N, int K, T alpha, const T *A, int lda, const T *X,
                       int incX, T beta, T *Y, int incY) {
  guarded(fn, [&] {
    row_major(order);
    nonneg(N, "N < 0");
    nonneg(K, "K < 0");
    if (N == 0) return;
    ld_ok(lda, long(K) + 1, "lda < K + 1");
    inc_ok(incX, "incX == 0");
    inc_ok(incY, "incY == 0");
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    Stager st;
    const T *dA = st.mat(A, N, long(K) + 1, lda, false);
    const T *dx = st.vec(X, N, incX, false);
    T *dy = st.vec(Y, N, incY, true);
    l2::sbmv<T>(Uplo == kUpper, N, K, alpha, dA, lda, dx, incX, beta, dy, incY);
    st.finish();
  });
}

// test/level2/stbmv/exo_stbmv.h and stbsv/exo_stbsv.h: Upper vs anything
// else, NoTrans vs anything else, unit diagonal only for CblasUnit.
template <typename T>
static void tb_entry(const char *fn, bool solve, int order, int Uplo, int TransA, int Diag, int N, int K, const T *A,
                     int lda, T *X, int incX) {
  guarded(fn, [&] {
    row_major(order);
    nonneg(N, "N < 0");
    nonneg(K, "K < 0");
    if (N == 0) return;
    ld_ok(lda, long(K) + 1, "lda < K + 1");
    inc_ok(incX, "incX == 0");
    X = rebase(X, N, incX);
    Stager st;
    const T *dA = st.mat(A, N, long(K) + 1, lda, false);
    T *dx = st.vec(X, N, incX, true);
    if (solve)
      l2::tbsv<T>(Uplo == kUpper, TransA != kNoTrans, Diag == kUnit, N, K, dA, lda, dx, incX);
    else
      l2::tbmv<T>(Uplo == kUpper, TransA != kNoTrans, Diag == kUnit, N, K, dA, lda, dx, incX);
    st.finish();
  });
}

// test/level3/syr2k/exo_syr2k_wrapper.h:9-32.  Uplo other than Upper or Lower
// leaves C unchanged, as neither branch of the proc's guard
// (src/level3/syr2k.py:33) and of trmscal (src/level3/mscal.py:26) holds.
template <typename T>
static void syr2k_entry(const char *fn, int Order, int Uplo, int Trans, int N, int K, T alpha, const T *A, int lda,
                        const T *B, int ldb, T beta, T *C, int ldc) {
  guarded(fn, [&] {
    row_major(Order);
    nonneg(N, "N < 0");
    nonneg(K, "K < 0");
    if (N == 0 || (Uplo != kUpper && Uplo != kLower)) return;
    const bool trans = Trans != kNoTrans;
    const long ar = trans ? K : N, ac = trans ? N : K;
    if (K > 0) {
      ld_ok(lda, ac, "lda too small");
      ld_ok(ldb, ac, "ldb too small");
    }
    ld_ok(ldc, N, "ldc < max(1, N)");
    Stager st;
    const T *dA = K > 0 ? st.mat(A, ar, ac, lda, false) : A;
    const T *dB = K > 0 ? st.mat(B, ar, ac, ldb, false) : B;
    T *dC = st.mat(C, N, N, ldc, true);
    syr2k_dispatch(Uplo == kUpper, trans, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc);
    st.finish();
  });
}

// test/level3/strmm/exo_strmm.h:7-58: Left only (the reference's Right
// branches are empty, so a row-major Right call leaves B unchanged); Diag is
// unit only when it equals CblasUnit.  right_ok: the column-major mapping
// of a Left call, B^T = alpha B^T op(A)^T, runs as a row-major Right call.
template <typename T>
static void trmm_entry(const char *fn, int Order, int Side, int Uplo, int TransA, int Diag, int M, int N, T alpha,
                       const T *A, int lda, T *B, int ldb, bool right_ok = false) {
  guarded(fn, [&] {
    row_major(Order);
    const bool left = Side == kLeft;
    if (!left && !right_ok) return;
    nonneg(M, "M < 0");
    nonneg(N, "N < 0");
    if (M == 0 || N == 0) return;
    const long ka = left ? M : N;  // A is ka x ka
    ld_ok(lda, ka, "lda < max(1, K)");
    ld_ok(ldb, N, "ldb < max(1, N)");
    Stager st;
    const T *dA = st.mat(A, ka, ka, lda, false);
    T *dB = st.mat(B, M, N, ldb, true);
    l3::trmm_simt<T>(left, Uplo == kUpper, TransA != kNoTrans, Diag == kUnit, M, N, alpha, dA, lda, dB, ldb);
    st.finish();
  });
}

// Column-major calls, when enabled (exoblas_set_column_major), are the
// row-major call on the transposed view of every operand: a column-major
// M x N matrix with leading dimension ld is the row-major N x M matrix with
// the same ld.  So gemm swaps (A, TransA) with (B, TransB) and M with N,
// gemv flips Trans and swaps M, N, ger swaps (X, M) with (Y, N), and the
// triangle of a symmetric or triangular operand changes sides: Uplo flips,
// with Trans (trmv/trsv/tbmv/tbsv/syrk/syr2k) or Side (symm/trmm) as the
// transposition requires.  By default a column-major call is rejected, as
// in the reference (e.g. test/level3/gemm/exo_gemm_wrapper.h:15-17).
static bool col_major(int order) { return order == kColMajor && column_major_enabled(); }
static CBLAS_TRANSPOSE flip_t(int t) { return CBLAS_TRANSPOSE(t == kNoTrans ? kTrans : kNoTrans); }
static CBLAS_UPLO flip_u(int u) { return CBLAS_UPLO(u == kUpper ? kLower : kUpper); }
static CBLAS_SIDE flip_s(int s) { return CBLAS_SIDE(s == kLeft ? kRight : kLeft); }

}  // namespace exb

using namespace exb;

extern "C" {

void exo_sgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE TransA, const int M, const int N,
               const float alpha, const float *A, const int lda, const float *X, const int incX, const float beta,
               float *Y, const int incY) {
  if (col_major(order)) return gemv_entry<float>("exo_sgemv", kRowMajor, flip_t(TransA), N, M, alpha, A, lda, X, incX, beta, Y, incY);
  gemv_entry<float>("exo_sgemv", order, TransA, M, N, alpha, A, lda, X, incX, beta, Y, incY);
}
void exo_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE TransA, const int M, const int N,
               const double alpha, const double *A, const int lda, const double *X, const int incX, const double beta,
               double *Y, const int incY) {
  if (col_major(order)) return gemv_entry<double>("exo_dgemv", kRowMajor, flip_t(TransA), N, M, alpha, A, lda, X, incX, beta, Y, incY);
  gemv_entry<double>("exo_dgemv", order, TransA, M, N, alpha, A, lda, X, incX, beta, Y, incY);
}
void exo_sger(const enum CBLAS_ORDER order, const int M, const int N, const float alpha, const float *X,
              const int incX, const float *Y, const int incY, float *A, const int lda) {
  if (col_major(order)) return ger_entry<float>("exo_sger", N, M, alpha, Y, incY, X, incX, A, lda);
  ger_entry<float>("exo_sger", M, N, alpha, X, incX, Y, incY, A, lda);
}
void exo_dger(const enum CBLAS_ORDER order, const int M, const int N, const double alpha, const double *X,
              const int incX, const double *Y, const int incY, double *A, const int lda) {
  if (col_major(order)) return ger_entry<double>("exo_dger", N, M, alpha, Y, incY, X, incX, A, lda);
  ger_entry<double>("exo_dger", M, N, alpha, X, incX, Y, incY, A, lda);
}
void exo_ssymv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const float alpha,
               const float *A, const int lda, const float *X, const int incX, const float beta, float *Y,
               const int incY) {
  if (col_major(order)) return symv_entry<float>("exo_ssymv", kRowMajor, flip_u(Uplo), N, alpha, A, lda, X, incX, beta, Y, incY);
  symv_entry<float>("exo_ssymv", order, Uplo, N, alpha, A, lda, X, incX, beta, Y, incY);
}
void exo_dsymv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const double alpha,
               const double *A, const int lda, const double *X, const int incX, const double beta, double *Y,
               const int incY) {
  if (col_major(order)) return symv_entry<double>("exo_dsymv", kRowMajor, flip_u(Uplo), N, alpha, A, lda, X, incX, beta, Y, incY);
  symv_entry<double>("exo_dsymv", order, Uplo, N, alpha, A, lda, X, incX, beta, Y, incY);
}
void exo_ssyr(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const float alpha,
              const float *X, const int incX, float *A, const int lda) {
  if (col_major(order)) return syr_entry<float>("exo_ssyr", kRowMajor, flip_u(Uplo), N, alpha, X, incX, A, lda);
  syr_entry<float>("exo_ssyr", order, Uplo, N, alpha, X, incX, A, lda);
}
void exo_dsyr(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const double alpha,
              const double *X, const int incX, double *A, const int lda) {
  if (col_major(order)) return syr_entry<double>("exo_dsyr", kRowMajor, flip_u(Uplo), N, alpha, X, incX, A, lda);
  syr_entry<double>("exo_dsyr", order, Uplo, N, alpha, X, incX, A, lda);
}
void exo_ssyr2(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const float alpha,
               const float *X, const int incX, const float *Y, const int incY, float *A, const int lda) {
  if (col_major(order)) return syr2_entry<float>("exo_ssyr2", flip_u(Uplo), N, alpha, X, incX, Y, incY, A, lda);
  syr2_entry<float>("exo_ssyr2", Uplo, N, alpha, X, incX, Y, incY, A, lda);
}
void exo_dsyr2(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const double alpha,
               const double *X, const int incX, const double *Y, const int incY, double *A, const int lda) {
  if (col_major(order)) return syr2_entry<double>("exo_dsyr2", flip_u(Uplo), N, alpha, X, incX, Y, incY, A, lda);
  syr2_entry<double>("exo_dsyr2", Uplo, N, alpha, X, incX, Y, incY, A, lda);
}
void exo_strmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const float *A, const int lda, float *X, const int incX) {
  if (col_major(order)) return tr_entry<float, false>("exo_strmv", kRowMajor, flip_u(Uplo), flip_t(TransA), Diag, N, A, lda, X, incX);
  tr_entry<float, false>("exo_strmv", order, Uplo, TransA, Diag, N, A, lda, X, incX);
}
void exo_dtrmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const double *A, const int lda, double *X, const int incX) {
  if (col_major(order)) return tr_entry<double, false>("exo_dtrmv", kRowMajor, flip_u(Uplo), flip_t(TransA), Diag, N, A, lda, X, incX);
  tr_entry<double, false>("exo_dtrmv", order, Uplo, TransA, Diag, N, A, lda, X, incX);
}
void exo_strsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const float *A, const int lda, float *X, const int incX) {
  if (col_major(order)) return tr_entry<float, true>("exo_strsv", kRowMajor, flip_u(Uplo), flip_t(TransA), Diag, N, A, lda, X, incX);
  tr_entry<float, true>("exo_strsv", order, Uplo, TransA, Diag, N, A, lda, X, incX);
}
void exo_dtrsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const double *A, const int lda, double *X, const int incX) {
  if (col_major(order)) return tr_entry<double, true>("exo_dtrsv", kRowMajor, flip_u(Uplo), flip_t(TransA), Diag, N, A, lda, X, incX);
  tr_entry<double, true>("exo_dtrsv", order, Uplo, TransA, Diag, N, A, lda, X, incX);
}

void exo_sgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TransA, const enum CBLAS_TRANSPOSE TransB,
               const int M, const int N, const int K, const float alpha, const float *A, const int lda,
               const float *B, const int ldb, const float beta, float *C, const int ldc) {
  if (col_major(Order)) return gemm_entry<float>("exo_sgemm", kRowMajor, TransB, TransA, N, M, K, alpha, B, ldb, A, lda, beta, C, ldc);
  gemm_entry<float>("exo_sgemm", Order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}
void exo_dgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TransA, const enum CBLAS_TRANSPOSE TransB,
               const int M, const int N, const int K, const double alpha, const double *A, const int lda,
               const double *B, const int ldb, const double beta, double *C, const int ldc) {
  if (col_major(Order)) return gemm_entry<double>("exo_dgemm", kRowMajor, TransB, TransA, N, M, K, alpha, B, ldb, A, lda, beta, C, ldc);
  gemm_entry<double>("exo_dgemm", Order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}
void exo_ssymm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo, const int M,
               const int N, const float alpha, const float *A, const int lda, const float *B, const int ldb,
               const float beta, float *C, const int ldc) {
  if (col_major(Order)) return symm_entry<float>("exo_ssymm", kRowMajor, flip_s(Side), flip_u(Uplo), N, M, alpha, A, lda, B, ldb, beta, C, ldc);
  symm_entry<float>("exo_ssymm", Order, Side, Uplo, M, N, alpha, A, lda, B, ldb, beta, C, ldc);
}
void exo_dsymm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo, const int M,
               const int N, const double alpha, const double *A, const int lda, const double *B, const int ldb,
               const double beta, double *C, const int ldc) {
  if (col_major(Order)) return symm_entry<double>("exo_dsymm", kRowMajor, flip_s(Side), flip_u(Uplo), N, M, alpha, A, lda, B, ldb, beta, C, ldc);
  symm_entry<double>("exo_dsymm", Order, Side, Uplo, M, N, alpha, A, lda, B, ldb, beta, C, ldc);
}
void exo_ssyrk(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans,
               const int N, const int K, const float alpha, const float *A, const int lda, const float beta, float *C,
               const int ldc) {
  if (col_major(Order)) return syrk_entry<float>("exo_ssyrk", kRowMajor, flip_u(Uplo), flip_t(Trans), N, K, alpha, A, lda, beta, C, ldc);
  syrk_entry<float>("exo_ssyrk", Order, Uplo, Trans, N, K, alpha, A, lda, beta, C, ldc);
}
void exo_dsyrk(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans,
               const int N, const int K, const double alpha, const double *A, const int lda, const double beta,
               double *C, const int ldc) {
  if (col_major(Order)) return syrk_entry<double>("exo_dsyrk", kRowMajor, flip_u(Uplo), flip_t(Trans), N, K, alpha, A, lda, beta, C, ldc);
  syrk_entry<double>("exo_dsyrk", Order, Uplo, Trans, N, K, alpha, A, lda, beta, C, ldc);
}
void exo_sgbmv(const int M, const int N, const int KL, const int KU, const float alpha, const float *A,
               const int lda, const float *X, const int incX, const float beta, float *Y, const int incY) {
  gbmv_entry<float>("exo_sgbmv", M, N, KL, KU, alpha, A, lda, X, incX, beta, Y, incY);
}
void exo_dgbmv(const int M, const int N, const int KL, const int KU, const double alpha, const double *A,
               const int lda, const double *X, const int incX, const double beta, double *Y, const int incY) {
  gbmv_entry<double>("exo_dgbmv", M, N, KL, KU, alpha, A, lda, X, incX, beta, Y, incY);
}
void exo_ssbmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const int K, const float alpha,
               const float *A, const int lda, const float *X, const int incX, const float beta, float *Y,
               const int incY) {
  if (col_major(order)) return sbmv_entry<float>("exo_ssbmv", kRowMajor, flip_u(Uplo), N, K, alpha, A, lda, X, incX, beta, Y, incY);
  sbmv_entry<float>("exo_ssbmv", order, Uplo, N, K, alpha, A, lda, X, incX, beta, Y, incY);
}
void exo_dsbmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const int K, const double alpha,
               const double *A, const int lda, const double *X, const int incX, const double beta, double *Y,
               const int incY) {
  if (col_major(order)) return sbmv_entry<double>("exo_dsbmv", kRowMajor, flip_u(Uplo), N, K, alpha, A, lda, X, incX, beta, Y, incY);
  sbmv_entry<double>("exo_dsbmv", order, Uplo, N, K, alpha, A, lda, X, incX, beta, Y, incY);
}
void exo_stbmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const int K, const float *A, const int lda, float *X,
               const int incX) {
  if (col_major(order)) return tb_entry<float>("exo_stbmv", false, kRowMajor, flip_u(Uplo), flip_t(TransA), Diag, N, K, A, lda, X, incX);
  tb_entry<float>("exo_stbmv", false, order, Uplo, TransA, Diag, N, K, A, lda, X, incX);
}
void exo_dtbmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const int K, const double *A, const int lda, double *X,
               const int incX) {
  if (col_major(order)) return tb_entry<double>("exo_dtbmv", false, kRowMajor, flip_u(Uplo), flip_t(TransA), Diag, N, K, A, lda, X, incX);
  tb_entry<double>("exo_dtbmv", false, order, Uplo, TransA, Diag, N, K, A, lda, X, incX);
}
void exo_stbsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const int K, const float *A, const int lda, float *X,
               const int incX) {
  if (col_major(order)) return tb_entry<float>("exo_stbsv", true, kRowMajor, flip_u(Uplo), flip_t(TransA), Diag, N, K, A, lda, X, incX);
  tb_entry<float>("exo_stbsv", true, order, Uplo, TransA, Diag, N, K, A, lda, X, incX);
}
void exo_dtbsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const int K, const double *A, const int lda, double *X,
               const int incX) {
  if (col_major(order)) return tb_entry<double>("exo_dtbsv", true, kRowMajor, flip_u(Uplo), flip_t(TransA), Diag, N, K, A, lda, X, incX);
  tb_entry<double>("exo_dtbsv", true, order, Uplo, TransA, Diag, N, K, A, lda, X, incX);
}
void exo_ssyr2k(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans,
                const int N, const int K, const float alpha, const float *A, const int lda, const float *B,
                const int ldb, const float beta, float *C, const int ldc) {
  if (col_major(Order)) return syr2k_entry<float>("exo_ssyr2k", kRowMajor, flip_u(Uplo), flip_t(Trans), N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  syr2k_entry<float>("exo_ssyr2k", Order, Uplo, Trans, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}
void exo_dsyr2k(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans,
                const int N, const int K, const double alpha, const double *A, const int lda, const double *B,
                const int ldb, const double beta, double *C, const int ldc) {
  if (col_major(Order)) return syr2k_entry<double>("exo_dsyr2k", kRowMajor, flip_u(Uplo), flip_t(Trans), N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  syr2k_entry<double>("exo_dsyr2k", Order, Uplo, Trans, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}
void exo_strmm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo,
               const enum CBLAS_TRANSPOSE TransA, const enum CBLAS_DIAG Diag, const int M, const int N,
               const float alpha, const float *A, const int lda, float *B, const int ldb) {
  if (col_major(Order)) return trmm_entry<float>("exo_strmm", kRowMajor, flip_s(Side), flip_u(Uplo), TransA, Diag, N, M, alpha, A, lda, B, ldb, true);
  trmm_entry<float>("exo_strmm", Order, Side, Uplo, TransA, Diag, M, N, alpha, A, lda, B, ldb);
}

}  // extern "C"
