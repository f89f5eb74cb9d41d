// CPU oracle for the exoblas_gb300 BLAS hot path. TEST INFRASTRUCTURE ONLY.
//
// This file restates, in plain C++, the algorithm of every in-scope ExoBLAS
// `@proc` (the unscheduled loop nest, in its loop order) together with the
// CBLAS-order wrapper that dispatches to it (flag checks, negative-increment
// rebasing, alpha/beta special cases, beta pre-scaling for level 3).  It is
// the checker for the GPU library and the CPU baseline timed beside it; it is
// never linked into, loaded by or called from the GPU library itself.
//
// Each function cites the reference file:line it follows.  Sources:
//   src/level1/{asum,axpy,dot,dsdot,exo_copy,rot,rotm,scal,swap}.py
//   src/level2/{gemv,ger,symv,syr,syr2,trmv,trsv}.py
//   src/level3/{gemm,symm,syrk,syr2k,trmm,mscal}.py, src/level2/{gbmv,sbmv,tbmv,tbsv}.py
//   test/level*/<op>/exo_<op>_wrapper.h, test/level1/sdsdot/exo_sdsdot.h
//
// The reference raises a C++ exception when Order != RowMajor.  The oracle
// records status 1 (read with oracle_last_status()) and returns instead.
//
// Also here: double-double reference kernels (TwoSum after Knuth, TwoProd via
// fma after Dekker 1971, Dot2 after Ogita, Rump and Oishi 2005) used as the
// high-precision oracle for d-precision results, and multi-threaded drivers
// of the same algorithms (row / range partitions over std::thread) used only
// to time the CPU baseline on all host cores.

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <thread>
#include <vector>

namespace {

// CBLAS flag values (src/common/cblas_enums.py:4-33, test/common/cblas.h:10-18)
constexpr int kRowMajor = 101;
constexpr int kNoTrans = 111;
constexpr int kUpper = 121;
constexpr int kLower = 122;
constexpr int kNonUnit = 131;
constexpr int kUnit = 132;
constexpr int kLeft = 141;

thread_local int g_status = 0;

inline bool row_major_or_fail(int order) {
  if (order != kRowMajor) {
    g_status = 1;
    return false;
  }
  return true;
}

// A strided 1-D window: element i lives at p[i * s] (s may be negative after
// the wrapper rebased the pointer, exactly as the reference wrappers do).
template <typename T>
struct Vec {
  T *p;
  long s;
  T &operator[](long i) const { return p[i * s]; }
};

// A row-major 2-D window with leading dimension ld and unit inner stride.
template <typename T>
struct Mat {
  T *p;
  long ld;
  T &operator()(long i, long j) const { return p[i * ld + j]; }
};

template <typename T>
T *rebase(T *x, int n, int inc) {
  // exo_axpy_wrapper.h:23-28 and every other wrapper: X + (1 - N) * incX
  return inc < 0 ? x + (long)(1 - n) * inc : x;
}

// ---------------------------------------------------------------- level 1 --

// src/level1/asum.py:11-15 (select(0, x, x, -x) == |x|)
template <typename T>
T asum_proc(long n, Vec<T> x) {
  T result = 0.0;
  for (long i = 0; i < n; ++i) result += (T(0) < x[i]) ? x[i] : -x[i];
  return result;
}

// test/level1/asum/exo_asum_wrapper.h:5-23 (incX < 0 returns 0)
template <typename T>
T asum_wrap(int N, const T *X, int incX) {
  g_status = 0;
  if (incX != 1 && incX < 0) return 0.0;
  return asum_proc<T>(N, Vec<T>{const_cast<T *>(X), incX});
}

// src/level1/axpy.py:9-19
template <typename T>
void axpy_proc(long n, T alpha, Vec<T> x, Vec<T> y) {
  for (long i = 0; i < n; ++i) y[i] += alpha * x[i];
}
template <typename T>
void axpy_alpha_1_proc(long n, Vec<T> x, Vec<T> y) {
  for (long i = 0; i < n; ++i) y[i] += x[i];
}

// test/level1/axpy/exo_axpy_wrapper.h:5-34
template <typename T>
void axpy_wrap(int N, T alpha, const T *X, int incX, T *Y, int incY) {
  g_status = 0;
  if (alpha == 0.0) return;
  if (incX == 1 && incY == 1) {
    if (alpha == 1.0)
      axpy_alpha_1_proc<T>(N, Vec<T>{const_cast<T *>(X), 1}, Vec<T>{Y, 1});
    else
      axpy_proc<T>(N, alpha, Vec<T>{const_cast<T *>(X), 1}, Vec<T>{Y, 1});
  } else {
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
    axpy_proc<T>(N, alpha, Vec<T>{const_cast<T *>(X), incX}, Vec<T>{Y, incY});
  }
}

// src/level1/dot.py:9-13
template <typename T>
T dot_proc(long n, Vec<T> x, Vec<T> y) {
  T result = 0.0;
  for (long i = 0; i < n; ++i) result += x[i] * y[i];
  return result;
}

// test/level1/dot/exo_dot_wrapper.h:5-27
template <typename T>
T dot_wrap(int N, const T *X, int incX, const T *Y, int incY) {
  g_status = 0;
  if (!(incX == 1 && incY == 1)) {
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
  }
  return dot_proc<T>(N, Vec<T>{const_cast<T *>(X), incX},
                     Vec<T>{const_cast<T *>(Y), incY});
}

// src/level1/dsdot.py:11-21
double dsdot_proc(long n, Vec<float> x, Vec<float> y) {
  double d_dot = 0.0;
  for (long i = 0; i < n; ++i) {
    double d_x = x[i];
    double d_y = y[i];
    d_dot += d_x * d_y;
  }
  return d_dot;
}

// src/level1/dsdot.py:24-36
float sdsdot_proc(long n, float sb, Vec<float> x, Vec<float> y) {
  double d_dot = dsdot_proc(n, x, y);
  double d_result = d_dot;
  d_result += sb;
  return (float)d_result;
}

// src/level1/exo_copy.py:9-12
template <typename T>
void copy_proc(long n, Vec<T> x, Vec<T> y) {
  for (long i = 0; i < n; ++i) y[i] = x[i];
}

// src/level1/swap.py:9-15
template <typename T>
void swap_proc(long n, Vec<T> x, Vec<T> y) {
  for (long i = 0; i < n; ++i) {
    T tmp = x[i];
    x[i] = y[i];
    y[i] = tmp;
  }
}

// src/level1/scal.py:9-19
template <typename T>
void scal_proc(long n, T alpha, Vec<T> x) {
  for (long i = 0; i < n; ++i) x[i] = alpha * x[i];
}
template <typename T>
void scal_alpha_0_proc(long n, Vec<T> x) {
  for (long i = 0; i < n; ++i) x[i] = 0.0;
}

// test/level1/scal/exo_scal_wrapper.h:7-35
template <typename T>
void scal_wrap(int N, T alpha, T *X, int incX) {
  g_status = 0;
  if (alpha == 1.0) return;
  if (incX != 1 && incX < 0) return;
  if (alpha == 0.0)
    scal_alpha_0_proc<T>(N, Vec<T>{X, incX});
  else
    scal_proc<T>(N, alpha, Vec<T>{X, incX});
}

// src/level1/rot.py:9-15
template <typename T>
void rot_proc(long n, Vec<T> x, Vec<T> y, T c, T s) {
  for (long i = 0; i < n; ++i) {
    T xReg = x[i];
    x[i] = c * xReg + s * y[i];
    y[i] = -s * xReg + c * y[i];
  }
}

// src/level1/rotm.py:9-33 with H = {P[1], P[3], P[2], P[4]} as a row-major
// 2x2 (test/level1/rotm/exo_rotm_wrapper.h:8); flags other than -1, 0, 1
// (e.g. -2) leave x and y untouched (exo_rotm_wrapper.h:10-22).
template <typename T>
void rotm_proc(long n, Vec<T> x, Vec<T> y, const T *P) {
  const T h00 = P[1], h01 = P[3], h10 = P[2], h11 = P[4];
  const T flag = P[0];
  for (long i = 0; i < n; ++i) {
    T xReg = x[i];
    if (flag == -1.0) {
      x[i] = h00 * xReg + h01 * y[i];
      y[i] = h10 * xReg + h11 * y[i];
    } else if (flag == 0.0) {
      x[i] = xReg + h01 * y[i];
      y[i] = h10 * xReg + y[i];
    } else if (flag == 1.0) {
      x[i] = h00 * xReg + y[i];
      y[i] = -xReg + h11 * y[i];
    } else {
      return;
    }
  }
}

template <typename T>
void two_vec_wrap_prep(int N, T *&X, int incX, T *&Y, int incY) {
  g_status = 0;
  if (!(incX == 1 && incY == 1)) {
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
  }
}

// ---------------------------------------------------------------- level 2 --

// src/level2/gemv.py:10-22; wrapper test/level2/gemv/exo_gemv_wrapper.h:7-39
template <typename T>
void gemv_wrap(int order, int TransA, int M, int N, T alpha, const T *A,
               int lda, const T *X, int incX, T beta, T *Y, int incY) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  const int m = TransA == kNoTrans ? M : N;  // length of y
  const int n = TransA == kNoTrans ? N : M;  // length of x
  if (!(incX == 1 && incY == 1)) {
    X = rebase(X, n, incX);
    Y = rebase(Y, m, incY);
  }
  Vec<T> x{const_cast<T *>(X), incX}, y{Y, incY};
  Mat<T> a{const_cast<T *>(A), lda};
  for (long i = 0; i < m; ++i) y[i] = y[i] * beta;
  if (TransA == kNoTrans) {
    for (long i = 0; i < m; ++i)
      for (long j = 0; j < n; ++j) y[i] += alpha * (x[j] * a(i, j));
  } else {
    // AT has shape [n, m] (the caller's M x N matrix)
    for (long i = 0; i < n; ++i)
      for (long j = 0; j < m; ++j) y[j] += alpha * x[i] * a(i, j);
  }
}

// src/level2/ger.py:9-15; wrapper test/level2/ger/exo_ger_wrapper.h:7-34
// (the wrapper does not check Order)
template <typename T>
void ger_wrap(int order, int M, int N, T alpha, const T *X, int incX,
              const T *Y, int incY, T *A, int lda) {
  (void)order;
  g_status = 0;
  if (alpha == 0.0) return;
  if (!(incX == 1 && incY == 1)) {
    X = rebase(X, M, incX);
    Y = rebase(Y, N, incY);
  }
  Vec<T> x{const_cast<T *>(X), incX}, y{const_cast<T *>(Y), incY};
  Mat<T> a{A, lda};
  for (long i = 0; i < M; ++i)
    for (long j = 0; j < N; ++j) a(i, j) += alpha * x[i] * y[j];
}

// src/level2/symv.py:10-35; wrapper test/level2/symv/exo_symv_wrapper.h:7-34
template <typename T>
void symv_wrap(int order, int Uplo, int N, T alpha, const T *A, int lda,
               const T *X, int incX, T beta, T *Y, int incY) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  X = rebase(X, N, incX);
  Y = rebase(Y, N, incY);
  Vec<T> x{const_cast<T *>(X), incX}, y{Y, incY};
  Mat<T> a{const_cast<T *>(A), lda};
  const long n = N;
  for (long i = 0; i < n; ++i) y[i] = beta * y[i];
  for (long i = 0; i < n; ++i) {
    if (Uplo == kUpper) {
      const long ii = n - i - 1;
      T temp = alpha * x[ii];
      T dot = 0.0;
      for (long j = 0; j < i + 1; ++j) {
        const long jj = n - j - 1;
        y[jj] += temp * a(ii, jj);
        dot += a(ii, jj) * x[jj];
      }
      y[ii] += alpha * (dot - a(ii, ii) * x[ii]);
    } else {
      T temp = alpha * x[i];
      T dot = 0.0;
      for (long j = 0; j < i + 1; ++j) {
        y[j] += temp * a(i, j);
        dot += a(i, j) * x[j];
      }
      y[i] += alpha * (dot - a(i, i) * x[i]);
    }
  }
}

// src/level2/syr.py:10-19; wrapper test/level2/syr/exo_syr_wrapper.h:5-32
template <typename T>
void syr_wrap(int order, int Uplo, int N, T alpha, const T *X, int incX, T *A,
              int lda) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  if (alpha == 0.0) return;
  if (incX != 1) X = rebase(X, N, incX);
  Vec<T> x{const_cast<T *>(X), incX};
  Mat<T> a{A, lda};
  const long n = N;
  for (long i = 0; i < n; ++i)
    for (long j = 0; j < i + 1; ++j) {
      if (Uplo == kUpper)
        a(n - i - 1, n - j - 1) += (alpha * x[n - i - 1]) * x[n - j - 1];
      else
        a(i, j) += alpha * x[i] * x[j];
    }
}

// src/level2/syr2.py:9-27; wrapper test/level2/syr2/exo_syr2_wrapper.h:5-36
// (the wrapper does not check Order)
template <typename T>
void syr2_wrap(int order, int Uplo, int N, T alpha, const T *X, int incX,
               const T *Y, int incY, T *A, int lda) {
  (void)order;
  g_status = 0;
  if (alpha == 0.0) return;
  X = rebase(X, N, incX);
  Y = rebase(Y, N, incY);
  Vec<T> x{const_cast<T *>(X), incX}, y{const_cast<T *>(Y), incY};
  Mat<T> a{A, lda};
  const long n = N;
  for (long i = 0; i < n; ++i)
    for (long j = 0; j < i + 1; ++j) {
      if (Uplo == kUpper) {
        const long ii = n - i - 1, jj = n - j - 1;
        a(ii, jj) += (alpha * x[ii]) * y[jj] + (alpha * y[ii]) * x[jj];
      } else {
        a(i, j) += (alpha * x[i]) * y[j] + (alpha * y[i]) * x[j];
      }
    }
}

// src/level2/trmv.py:9-43; wrapper test/level2/trmv/exo_trmv_wrapper.h:7-29
template <typename T>
void trmv_wrap(int order, int Uplo, int TransA, int Diag, int N, const T *A,
               int lda, T *X, int incX) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  X = rebase(X, N, incX);
  Vec<T> x{X, incX};
  Mat<T> a{const_cast<T *>(A), lda};
  const long n = N;
  std::vector<T> xCopy(n > 0 ? n : 0, T(0));
  for (long i = 0; i < n; ++i) {
    if (TransA == kNoTrans) {
      if (Uplo == kUpper) {
        const long ii = n - i - 1;
        for (long j = 0; j < i + 1; ++j)
          xCopy[ii] += a(ii, n - j - 1) * x[n - j - 1];
        if (Diag == kUnit) xCopy[ii] += (1 - a(ii, ii)) * x[ii];
      } else {
        for (long j = 0; j < i + 1; ++j) xCopy[i] += a(i, j) * x[j];
        if (Diag == kUnit) xCopy[i] += (1 - a(i, i)) * x[i];
      }
    } else {
      if (Uplo == kUpper) {
        const long ii = n - i - 1;
        for (long j = 0; j < i + 1; ++j)
          xCopy[n - j - 1] += a(ii, n - j - 1) * x[ii];
        if (Diag == kUnit) xCopy[ii] += (1 - a(ii, ii)) * x[ii];
      } else {
        for (long j = 0; j < i + 1; ++j) xCopy[j] += a(i, j) * x[i];
        if (Diag == kUnit) xCopy[i] += (1 - a(i, i)) * x[i];
      }
    }
  }
  for (long l = 0; l < n; ++l) x[l] = xCopy[l];
}

// src/level2/trsv.py:10-52; wrapper test/level2/trsv/exo_trsv_wrapper.h:7-29
template <typename T>
void trsv_wrap(int order, int Uplo, int TransA, int Diag, int N, const T *A,
               int lda, T *X, int incX) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  X = rebase(X, N, incX);
  Vec<T> x{X, incX};
  Mat<T> a{const_cast<T *>(A), lda};
  const long n = N;
  std::vector<T> Dot(n > 0 ? n : 0, T(0));
  for (long i = 0; i < n; ++i) {
    if (TransA == kNoTrans) {
      T dot = 0.0;
      if (Uplo == kUpper) {
        const long ii = n - i - 1;
        for (long j = 0; j < i; ++j) dot += a(ii, n - j - 1) * x[n - j - 1];
        x[ii] = x[ii] - dot;
        if (Diag == kNonUnit) x[ii] = x[ii] / a(ii, ii);
      } else {
        for (long j = 0; j < i; ++j) dot += a(i, j) * x[j];
        x[i] = x[i] - dot;
        if (Diag == kNonUnit) x[i] = x[i] / a(i, i);
      }
    } else {
      if (Uplo == kUpper) {
        x[i] = x[i] - Dot[i];
        if (Diag == kNonUnit) x[i] = x[i] / a(i, i);
        for (long j = 0; j < n - i - 1; ++j)
          Dot[n - j - 1] += a(i, n - j - 1) * x[i];
      } else {
        const long ii = n - i - 1;
        x[ii] = x[ii] - Dot[ii];
        if (Diag == kNonUnit) x[ii] = x[ii] / a(ii, ii);
        for (long j = 0; j < n - i - 1; ++j) Dot[j] += a(ii, j) * x[ii];
      }
    }
  }
}

// ---------------------------------------------------------------- level 3 --

// src/level3/mscal.py:12-18 (full matrix) and :21-28 (one triangle)
template <typename T>
void mscal_proc(long M, long N, T beta, Mat<T> c) {
  for (long i = 0; i < M; ++i)
    for (long j = 0; j < N; ++j) c(i, j) = c(i, j) * beta;
}
template <typename T>
void trmscal_proc(int Uplo, long N, T beta, Mat<T> c) {
  for (long i = 0; i < N; ++i)
    for (long j = 0; j < N; ++j)
      if ((Uplo == kUpper && j >= i) || (Uplo == kLower && j < i + 1))
        c(i, j) = c(i, j) * beta;
}

// src/level3/gemm.py:17-47 over the row range [i0, i1).  Per element of C the
// k-sum runs in increasing k exactly as in the i,j,k nest; the i,k,j order
// used here only changes which element is touched next, not the sum order.
template <typename T>
void gemm_rows(int TransA, int TransB, long i0, long i1, long N, long K,
               T alpha, Mat<T> a, Mat<T> b, Mat<T> c) {
  for (long i = i0; i < i1; ++i) {
    T *ci = &c(i, 0);
    if (TransB == kNoTrans) {
      for (long k = 0; k < K; ++k) {
        const T aik = TransA == kNoTrans ? a(i, k) : a(k, i);
        const T *bk = &b(k, 0);
        for (long j = 0; j < N; ++j) ci[j] += alpha * (aik * bk[j]);
      }
    } else {
      for (long j = 0; j < N; ++j) {
        T acc = ci[j];
        const T *bj = &b(j, 0);
        for (long k = 0; k < K; ++k) {
          const T aik = TransA == kNoTrans ? a(i, k) : a(k, i);
          acc += alpha * (aik * bj[k]);
        }
        ci[j] = acc;
      }
    }
  }
}

// test/level3/gemm/exo_gemm_wrapper.h:9-28: C *= beta (mscal), then the proc
template <typename T>
void gemm_wrap(int order, int TransA, int TransB, int M, int N, int K,
               T alpha, const T *A, int lda, const T *B, int ldb, T beta, T *C,
               int ldc) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  Mat<T> a{const_cast<T *>(A), lda}, b{const_cast<T *>(B), ldb}, c{C, ldc};
  mscal_proc<T>(M, N, beta, c);
  gemm_rows<T>(TransA, TransB, 0, M, N, K, alpha, a, b, c);
}

// src/level3/symm.py:16-47 over the row range [i0, i1)
template <typename T>
void symm_rows(int Side, int Uplo, long i0, long i1, long M, long N, T alpha,
               Mat<T> a, Mat<T> b, Mat<T> c) {
  for (long i = i0; i < i1; ++i) {
    T *ci = &c(i, 0);
    if (Side == kLeft) {
      for (long k = 0; k < M; ++k) {
        T a_val;
        if (Uplo == kUpper)
          a_val = k < i + 1 ? a(k, i) : a(i, k);
        else
          a_val = k < i + 1 ? a(i, k) : a(k, i);
        const T *bk = &b(k, 0);
        for (long j = 0; j < N; ++j) ci[j] += alpha * (a_val * bk[j]);
      }
    } else {
      for (long k = 0; k < N; ++k) {
        const T bik = b(i, k);
        for (long j = 0; j < N; ++j) {
          T a_val;
          if (Uplo == kUpper)
            a_val = j < k + 1 ? a(j, k) : a(k, j);
          else
            a_val = j < k + 1 ? a(k, j) : a(j, k);
          ci[j] += alpha * (bik * a_val);
        }
      }
    }
  }
}

// test/level3/symm/exo_symm_wrapper.h:9-27
template <typename T>
void symm_wrap(int order, int Side, int Uplo, int M, int N, T alpha,
               const T *A, int lda, const T *B, int ldb, T beta, T *C,
               int ldc) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  Mat<T> a{const_cast<T *>(A), lda}, b{const_cast<T *>(B), ldb}, c{C, ldc};
  mscal_proc<T>(M, N, beta, c);
  symm_rows<T>(Side, Uplo, 0, M, M, N, alpha, a, b, c);
}

// src/level3/syrk.py:17-32 over the row range [i0, i1)
template <typename T>
void syrk_rows(int Uplo, int Trans, long i0, long i1, long N, long K, T alpha,
               Mat<T> a, Mat<T> c) {
  for (long i = i0; i < i1; ++i) {
    const long j0 = Uplo == kUpper ? i : 0;
    const long j1 = Uplo == kUpper ? N : i + 1;
    T *ci = &c(i, 0);
    if (Trans == kNoTrans) {
      const T *ai = &a(i, 0);
      for (long j = j0; j < j1; ++j) {
        const T *aj = &a(j, 0);
        T acc = ci[j];
        for (long k = 0; k < K; ++k) acc += alpha * (ai[k] * aj[k]);
        ci[j] = acc;
      }
    } else {
      for (long k = 0; k < K; ++k) {
        const T aki = a(k, i);
        const T *ak = &a(k, 0);
        for (long j = j0; j < j1; ++j) ci[j] += alpha * (aki * ak[j]);
      }
    }
  }
}

// test/level3/syrk/exo_syrk_wrapper.h:9-28: trmscal then the proc
template <typename T>
void syrk_wrap(int order, int Uplo, int Trans, int N, int K, T alpha,
               const T *A, int lda, T beta, T *C, int ldc) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  Mat<T> a{const_cast<T *>(A), lda}, c{C, ldc};
  trmscal_proc<T>(Uplo, N, beta, c);
  syrk_rows<T>(Uplo, Trans, 0, N, N, K, alpha, a, c);
}

// --------------------------------------------------------- nrm2, iamax --
// No reference counterpart (README.md:15).  nrm2: the two-pass scaled sum
// of squares (scale = max |x_i|, then scale * sqrt(sum (x_i / scale)^2)),
// free of overflow and underflow, over any increment (a negative one walks
// the vector backwards, 0 repeats x[0]) as in reference BLAS 3.10 and
// OpenBLAS; iamax: the reference BLAS loop (0 for N < 1 or incX < 1; start
// from |x[0]|, take an element only when strictly larger), 0-based.
template <typename T>
T nrm2_ref(int N, const T *X, int incX) {
  g_status = 0;
  if (N < 1) return T(0);
  if (incX < 0) X = X + long(1 - N) * incX;  // any increment, as the current reference BLAS
  double scale = 0;
  bool nan = false;
  for (long i = 0; i < N; ++i) {
    const double v = std::fabs(double(X[i * incX]));
    if (v != v) nan = true;
    if (v > scale) scale = v;
  }
  if (nan) return T(NAN);
  if (scale == 0 || std::isinf(scale)) return T(scale);
  double ss = 0;
  for (long i = 0; i < N; ++i) {
    const double v = double(X[i * incX]) / scale;
    ss += v * v;
  }
  return T(scale * std::sqrt(ss));
}
template <typename T>
long iamax_ref(int N, const T *X, int incX) {
  g_status = 0;
  if (N < 1 || incX < 1) return 0;
  long best = 0;
  T mx = std::fabs(X[0]);
  for (long i = 1; i < N; ++i) {
    const T v = std::fabs(X[i * incX]);
    if (v > mx) {
      mx = v;
      best = i;
    }
  }
  return best;
}

// ------------------------------------------------------- banded level 2 --
// Vec<T>: element i at p[i * inc] (the wrapper has already rebased p).

// src/level2/gbmv.py:12-50 (the proc leaves `result` unset for rows below
// the band's last column; here it is 0, so y[i] = beta y[i] as in CBLAS)
template <typename T>
void gbmv_proc(long m, long n, long kl, long ku, T alpha, T beta, Mat<T> a, const T *x, long incx, T *y, long incy) {
  for (long i = 0; i < m; ++i) {
    T result = 0;
    if (i - kl >= 0) {
      if (i + ku < n) {
        for (long j = 0; j < kl + ku + 1; ++j) result += a(i, j) * x[(i + (j - kl)) * incx];
      } else if (kl + n - i > 0) {
        for (long j = 0; j < kl + n - i; ++j) result += a(i, j) * x[(i + (j - kl)) * incx];
      }
    } else {
      if (i + ku < n) {
        for (long j = 0; j < i + ku + 1; ++j) result += a(i, kl - i + j) * x[j * incx];
      } else {
        for (long j = 0; j < n; ++j) result += a(i, kl - i + j) * x[j * incx];
      }
    }
    y[i * incy] = beta * y[i * incy] + alpha * result;
  }
}

// test/level2/sgbmv/exo_sgbmv.h:5-23.  That wrapper does not rebase negative
// increments (it would read before X); here they follow the CBLAS rule.
template <typename T>
void gbmv_wrap(int M, int N, int KL, int KU, T alpha, const T *A, int lda, const T *X, int incX, T beta, T *Y,
               int incY) {
  g_status = 0;
  if (incX < 0) X = X + long(1 - N) * incX;
  if (incY < 0) Y = Y + long(1 - M) * incY;
  gbmv_proc<T>(M, N, KL, KU, alpha, beta, Mat<T>{const_cast<T *>(A), lda}, X, incX, Y, incY);
}

// src/level2/sbmv.py:8-44 and test/level2/ssbmv/exo_ssbmv.h:7-52
template <typename T>
void sbmv_wrap(int order, int Uplo, int N, int K, T alpha, const T *A, int lda, const T *X, int incX, T beta, T *Y,
               int incY) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  if (incX < 0) X = X + long(1 - N) * incX;
  if (incY < 0) Y = Y + long(1 - N) * incY;
  Mat<T> a{const_cast<T *>(A), lda};
  auto x = [&](long i) -> T { return X[i * incX]; };
  auto y = [&](long i) -> T & { return Y[i * incY]; };
  if (beta != T(1))
    for (long i = 0; i < N; ++i) y(i) = beta * y(i);
  for (long i = 0; i < N; ++i) {
    const T temp = alpha * x(i);
    T dot = 0;
    if (Uplo == kUpper) {
      for (long j = 0; j < K; ++j)
        if (i + j + 1 < N) {
          y(i + j + 1) += temp * a(i, j + 1);
          dot += a(i, j + 1) * x(i + j + 1);
        }
      y(i) += temp * a(i, 0) + alpha * dot;
    } else {
      for (long j = 0; j < K; ++j)
        if (i - j - 1 >= 0) {
          y(i - j - 1) += temp * a(i, K - j - 1);
          dot += a(i, K - j - 1) * x(i - j - 1);
        }
      y(i) += temp * a(i, K) + alpha * dot;
    }
  }
}

// src/level2/tbmv.py:9-120 (the four procs in their loop order)
template <typename T>
void tbmv_proc(bool upper, bool trans, bool unit, long n, long k, Mat<T> a, T *X, long inc) {
  auto x = [&](long i) -> T & { return X[i * inc]; };
  if (!trans) {
    if (upper) {
      for (long i = 0; i < n - k; ++i) {
        T dot = unit ? x(i) : x(i) * a(i, 0);
        for (long j = 0; j < k; ++j) dot += a(i, j + 1) * x(i + j + 1);
        x(i) = dot;
      }
      for (long i = 0; i < k; ++i) {
        const long r = n - k + i;
        T dot = unit ? x(r) : x(r) * a(r, 0);
        for (long j = 0; j < k - i - 1; ++j) dot += a(r, j + 1) * x(r + j + 1);
        x(r) = dot;
      }
    } else {
      for (long i = 0; i < n - k; ++i) {
        const long r = n - i - 1;
        T dot = 0;
        for (long j = 0; j < k; ++j) dot += a(r, k - j - 1) * x(r - j - 1);
        dot += unit ? x(r) : x(r) * a(r, k);
        x(r) = dot;
      }
      for (long i = 0; i < k; ++i) {
        const long r = k - i - 1;
        T dot = 0;
        for (long j = 0; j < k - i - 1; ++j) dot += a(r, k - j - 1) * x(r - j - 1);
        dot += unit ? x(r) : x(r) * a(r, k);
        x(r) = dot;
      }
    }
    return;
  }
  std::vector<T> res(size_t(n), T(0));
  if (upper) {
    for (long i = 0; i < n - k; ++i) {
      res[i] += unit ? x(i) : x(i) * a(i, 0);
      for (long j = 0; j < k; ++j) res[i + j + 1] += a(i, j + 1) * x(i);
    }
    for (long i = 0; i < k; ++i) {
      const long r = n - k + i;
      res[r] += unit ? x(r) : x(r) * a(r, 0);
      for (long j = 0; j < k - i - 1; ++j) res[r + j + 1] += a(r, j + 1) * x(r);
    }
  } else {
    for (long i = 0; i < n - k; ++i) {
      const long r = n - i - 1;
      for (long j = 0; j < k; ++j) res[r - j - 1] += a(r, k - j - 1) * x(r);
      res[r] += unit ? x(r) : x(r) * a(r, k);
    }
    for (long i = 0; i < k; ++i) {
      const long r = k - i - 1;
      for (long j = 0; j < k - i - 1; ++j) res[r - j - 1] += a(r, k - j - 1) * x(r);
      res[r] += unit ? x(r) : x(r) * a(r, k);
    }
  }
  for (long i = 0; i < n; ++i) x(i) = res[i];
}

// src/level2/tbsv.py:9-120 (the four procs in their loop order)
template <typename T>
void tbsv_proc(bool upper, bool trans, bool unit, long n, long k, Mat<T> a, T *X, long inc) {
  auto x = [&](long i) -> T & { return X[i * inc]; };
  if (!trans && upper) {
    for (long i = 0; i < k; ++i) {
      const long r = n - i - 1;
      const T pivot = unit ? T(1) : a(r, 0);
      T dot = 0;
      for (long j = 0; j < i; ++j) dot += a(r, j + 1) * x(n - i + j);
      x(r) = (x(r) - dot) / pivot;
    }
    for (long i = 0; i < n - k; ++i) {
      const long r = n - (k + i) - 1;
      const T pivot = unit ? T(1) : a(r, 0);
      T dot = 0;
      for (long j = 0; j < k; ++j) dot += a(r, j + 1) * x(n - (k + i) + j);
      x(r) = (x(r) - dot) / pivot;
    }
  } else if (!trans) {
    for (long i = 0; i < k; ++i) {
      T dot = 0;
      for (long j = 0; j < i; ++j) dot += a(i, k - j - 1) * x(i - j - 1);
      const T pivot = unit ? T(1) : a(i, k);
      x(i) = (x(i) - dot) / pivot;
    }
    for (long i = 0; i < n - k; ++i) {
      T dot = 0;
      for (long j = 0; j < k; ++j) dot += a(i + k, k - j - 1) * x(i + k - j - 1);
      const T pivot = unit ? T(1) : a(i + k, k);
      x(i + k) = (x(i + k) - dot) / pivot;
    }
  } else if (upper) {
    for (long i = 0; i < n; ++i) {
      T dot = 0;
      for (long j = 0; j < k; ++j)
        if (i - j - 1 >= 0) dot += a(i - j - 1, j + 1) * x(i - j - 1);
      const T pivot = unit ? T(1) : a(i, 0);
      x(i) = (x(i) - dot) / pivot;
    }
  } else {
    for (long i = 0; i < n; ++i) {
      const T pivot = unit ? T(1) : a(n - i - 1, k);
      T dot = 0;
      for (long j = 0; j < k; ++j)
        if (n - i + j < n) dot += a(n - i + j, k - j - 1) * x(n - i + j);
      x(n - i - 1) = (x(n - i - 1) - dot) / pivot;
    }
  }
}

// test/level2/stbmv/exo_stbmv.h, test/level2/stbsv/exo_stbsv.h
template <typename T>
void tb_wrap(bool solve, int order, int Uplo, int TransA, int Diag, int N, int K, const T *A, int lda, T *X,
             int incX) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  if (incX < 0) X = X + long(1 - N) * incX;
  Mat<T> a{const_cast<T *>(A), lda};
  if (solve)
    tbsv_proc<T>(Uplo == kUpper, TransA != kNoTrans, Diag == kUnit, N, K, a, X, incX);
  else
    tbmv_proc<T>(Uplo == kUpper, TransA != kNoTrans, Diag == kUnit, N, K, a, X, incX);
}

// src/level3/syr2k.py:14-37: C[i,j] += alpha * (A[i,k] B[j,k] + B[i,k] A[j,k])
// over the stored triangle (NoTrans), with A^T / B^T read as AT[k,i] (Trans)
template <typename T>
void syr2k_rows(int Uplo, int Trans, long i0, long i1, long N, long K, T alpha, Mat<T> a, Mat<T> b, Mat<T> c) {
  if (Uplo != kUpper && Uplo != kLower) return;  // neither branch of the proc's guard
  for (long i = i0; i < i1; ++i) {
    const long j0 = Uplo == kUpper ? i : 0;
    const long j1 = Uplo == kUpper ? N : i + 1;
    for (long j = j0; j < j1; ++j) {
      T acc = c(i, j);
      for (long k = 0; k < K; ++k) {
        if (Trans == kNoTrans)
          acc += alpha * (a(i, k) * b(j, k) + b(i, k) * a(j, k));
        else
          acc += alpha * (a(k, i) * b(k, j) + b(k, i) * a(k, j));
      }
      c(i, j) = acc;
    }
  }
}

// test/level3/syr2k/exo_syr2k_wrapper.h:9-32: trmscal then the proc
template <typename T>
void syr2k_wrap(int order, int Uplo, int Trans, int N, int K, T alpha, const T *A, int lda, const T *B, int ldb,
                T beta, T *C, int ldc) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  Mat<T> a{const_cast<T *>(A), lda}, b{const_cast<T *>(B), ldb}, c{C, ldc};
  trmscal_proc<T>(Uplo, N, beta, c);
  syr2k_rows<T>(Uplo, Trans, 0, N, N, K, alpha, a, b, c);
}

// src/level3/trmm.py:12-78, the four Left procs exactly in their loop order
// (unit diagonal when `unit`); B = alpha op(A) B in place.
template <typename T>
void trmm_left(bool upper, bool trans, bool unit, long m, long n, T alpha, Mat<T> a, Mat<T> b) {
  const bool forward = upper != trans;  // Upper/NonTrans and Lower/Trans walk i upwards
  for (long j = 0; j < n; ++j) {
    for (long i = 0; i < m; ++i) {
      if (forward) {
        if (!unit) b(i, j) = a(i, i) * b(i, j);
        for (long k = 0; k < m - i - 1; ++k) {
          const T aik = upper ? a(i, i + k + 1) : a(i + k + 1, i);
          b(i, j) += aik * b(i + k + 1, j);
        }
        b(i, j) = alpha * b(i, j);
      } else {
        const long r = m - i - 1;
        const T org = b(r, j);
        b(r, j) = T(0);
        for (long k = 0; k < r; ++k) {
          const T ark = upper ? a(k, r) : a(r, k);
          b(r, j) += ark * b(k, j);
        }
        if (!unit)
          b(r, j) += a(r, r) * org;
        else
          b(r, j) += org;
        b(r, j) = alpha * b(r, j);
      }
    }
  }
}

// test/level3/strmm/exo_strmm.h:7-58: Left dispatches on Uplo / TransA; the
// Right side does nothing; Diag is unit only when it equals CblasUnit.
template <typename T>
void trmm_wrap(int order, int Side, int Uplo, int TransA, int Diag, int M, int N, T alpha, const T *A, int lda, T *B,
               int ldb) {
  g_status = 0;
  if (!row_major_or_fail(order)) return;
  if (Side != kLeft) return;
  Mat<T> a{const_cast<T *>(A), lda}, b{B, ldb};
  trmm_left<T>(Uplo == kUpper, TransA != kNoTrans, Diag == kUnit, M, N, alpha, a, b);
}

// --------------------------------------------------- double-double oracle --
// TwoSum (Knuth, TAOCP vol. 2), TwoProd through fma (Dekker 1971),
// Dot2 (Ogita, Rump, Oishi, "Accurate sum and dot product", SISC 2005).

struct DD {
  double hi, lo;
};
inline void two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  double z = s - a;
  e = (a - (s - z)) + (b - z);
}
inline void two_prod(double a, double b, double &p, double &e) {
  p = a * b;
  e = std::fma(a, b, -p);
}
inline void dd_add_prod(DD &acc, double a, double b) {
  double p, pe, s, se;
  two_prod(a, b, p, pe);
  two_sum(acc.hi, p, s, se);
  acc.hi = s;
  acc.lo += pe + se;
}
inline DD dd_norm(DD v) {
  double s, e;
  two_sum(v.hi, v.lo, s, e);
  return DD{s, e};
}

// ------------------------------------------- double-word arithmetic type --
// Dw is a number type with about 104 significand bits, so the restatements
// above can be instantiated with T = Dw and give the same loop nest evaluated
// in double-word arithmetic: the high-precision reference for d-precision
// results.  Algorithms from Joldes, Muller and Popescu, "Tight and rigorous
// error bounds for basic building blocks of double-word arithmetic", ACM TOMS
// 44(2), 2017: sum of two double-words (their Algorithm 6, relative error
// below 3u^2), product (Algorithm 12, below 5u^2) and a quotient by one
// correction step of the high-part quotient (below 2^-100 relative).  Inputs
// enter as {x, 0}, so every input is exact.  A non-finite high part wins
// over the low part when results are read back (Dw::value()).

inline void fast_two_sum(double a, double b, double &s, double &e) {
  s = a + b;
  e = b - (s - a);
}

struct Dw {
  double hi = 0.0, lo = 0.0;
  Dw() = default;
  Dw(double v) : hi(v), lo(0.0) {}  // NOLINT: implicit, like a double literal
  Dw(double h, double l) : hi(h), lo(l) {}
  double value() const { return std::isfinite(hi) ? hi + lo : hi; }
};
static_assert(sizeof(Dw) == 2 * sizeof(double), "Dw is two packed doubles");

inline Dw operator+(Dw x, Dw y) {
  if (!std::isfinite(x.hi) || !std::isfinite(y.hi)) return Dw(x.hi + y.hi);
  double sh, sl, th, tl, vh, vl, zh, zl;
  two_sum(x.hi, y.hi, sh, sl);
  two_sum(x.lo, y.lo, th, tl);
  const double c = sl + th;
  fast_two_sum(sh, c, vh, vl);
  const double w = tl + vl;
  fast_two_sum(vh, w, zh, zl);
  return Dw(zh, zl);
}
inline Dw operator-(Dw x) { return Dw(-x.hi, -x.lo); }
inline Dw operator-(Dw x, Dw y) { return x + (-y); }
inline Dw operator*(Dw x, Dw y) {
  double ch, cl1;
  two_prod(x.hi, y.hi, ch, cl1);
  if (!std::isfinite(ch) || ch == 0.0) return Dw(ch);
  const double tl0 = x.lo * y.lo;
  const double tl1 = std::fma(x.hi, y.lo, tl0);
  const double cl2 = std::fma(x.lo, y.hi, tl1);
  const double cl3 = cl1 + cl2;
  double zh, zl;
  fast_two_sum(ch, cl3, zh, zl);
  return Dw(zh, zl);
}
inline Dw operator/(Dw x, Dw y) {
  const double q1 = x.hi / y.hi;
  if (!std::isfinite(q1) || q1 == 0.0) return Dw(q1);
  const Dw r = x - y * Dw(q1);
  const double q2 = r.hi / y.hi;
  const Dw r2 = r - y * Dw(q2);
  const double q3 = r2.hi / y.hi;
  double s, e;
  fast_two_sum(q1, q2, s, e);
  return Dw(s, e) + Dw(q3);
}
inline Dw &operator+=(Dw &x, Dw y) { return x = x + y; }
inline Dw &operator-=(Dw &x, Dw y) { return x = x - y; }
inline Dw &operator*=(Dw &x, Dw y) { return x = x * y; }
inline bool operator==(Dw x, Dw y) { return x.hi == y.hi && x.lo == y.lo; }
inline bool operator!=(Dw x, Dw y) { return !(x == y); }
inline bool operator<(Dw x, Dw y) { return x.hi < y.hi || (x.hi == y.hi && x.lo < y.lo); }
inline bool operator>(Dw x, Dw y) { return y < x; }

// ------------------------------------------------------ threaded drivers --

template <typename F>
void parallel_for(int nthreads, long n, F f) {
  if (nthreads <= 1 || n < 2) {
    f(0, 0, n);
    return;
  }
  if (nthreads > n) nthreads = (int)n;
  std::vector<std::thread> th;
  th.reserve(nthreads);
  for (int t = 0; t < nthreads; ++t) {
    long lo = n * t / nthreads, hi = n * (t + 1) / nthreads;
    th.emplace_back([=] { f(t, lo, hi); });
  }
  for (auto &x : th) x.join();
}

}  // namespace

// ------------------------------------------------------------ C interface --

#define ORACLE_API extern "C" __attribute__((visibility("default")))

ORACLE_API int oracle_last_status(void) { return g_status; }

ORACLE_API float oracle_sasum(int N, const float *X, int incX) { return asum_wrap<float>(N, X, incX); }
ORACLE_API double oracle_dasum(int N, const double *X, int incX) { return asum_wrap<double>(N, X, incX); }

ORACLE_API void oracle_saxpy(int N, float alpha, const float *X, int incX, float *Y, int incY) { axpy_wrap<float>(N, alpha, X, incX, Y, incY); }
ORACLE_API void oracle_daxpy(int N, double alpha, const double *X, int incX, double *Y, int incY) { axpy_wrap<double>(N, alpha, X, incX, Y, incY); }

ORACLE_API float oracle_sdot(int N, const float *X, int incX, const float *Y, int incY) { return dot_wrap<float>(N, X, incX, Y, incY); }
ORACLE_API double oracle_ddot(int N, const double *X, int incX, const double *Y, int incY) { return dot_wrap<double>(N, X, incX, Y, incY); }

// test/level1/dsdot/exo_dsdot_wrapper.h:5-25
ORACLE_API double oracle_dsdot(int N, const float *X, int incX, const float *Y, int incY) {
  g_status = 0;
  if (!(incX == 1 && incY == 1)) {
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
  }
  return dsdot_proc(N, Vec<float>{const_cast<float *>(X), incX}, Vec<float>{const_cast<float *>(Y), incY});
}
// test/level1/sdsdot/exo_sdsdot.h:5-26
ORACLE_API float oracle_sdsdot(int N, float alpha, const float *X, int incX, const float *Y, int incY) {
  g_status = 0;
  if (!(incX == 1 && incY == 1)) {
    X = rebase(X, N, incX);
    Y = rebase(Y, N, incY);
  }
  return sdsdot_proc(N, alpha, Vec<float>{const_cast<float *>(X), incX}, Vec<float>{const_cast<float *>(Y), incY});
}

// test/level1/copy/exo_copy_wrapper.h:5-23
ORACLE_API void oracle_scopy(int N, const float *X, int incX, float *Y, int incY) {
  float *x = const_cast<float *>(X);
  two_vec_wrap_prep<float>(N, x, incX, Y, incY);
  copy_proc<float>(N, Vec<float>{x, incX}, Vec<float>{Y, incY});
}
ORACLE_API void oracle_dcopy(int N, const double *X, int incX, double *Y, int incY) {
  double *x = const_cast<double *>(X);
  two_vec_wrap_prep<double>(N, x, incX, Y, incY);
  copy_proc<double>(N, Vec<double>{x, incX}, Vec<double>{Y, incY});
}
// test/level1/swap/exo_swap_wrapper.h:5-23
ORACLE_API void oracle_sswap(int N, float *X, int incX, float *Y, int incY) {
  two_vec_wrap_prep<float>(N, X, incX, Y, incY);
  swap_proc<float>(N, Vec<float>{X, incX}, Vec<float>{Y, incY});
}
ORACLE_API void oracle_dswap(int N, double *X, int incX, double *Y, int incY) {
  two_vec_wrap_prep<double>(N, X, incX, Y, incY);
  swap_proc<double>(N, Vec<double>{X, incX}, Vec<double>{Y, incY});
}
ORACLE_API void oracle_sscal(int N, float alpha, float *X, int incX) { scal_wrap<float>(N, alpha, X, incX); }
ORACLE_API void oracle_dscal(int N, double alpha, double *X, int incX) { scal_wrap<double>(N, alpha, X, incX); }
// test/level1/rot/exo_rot_wrapper.h:5-23
ORACLE_API void oracle_srot(int N, float *X, int incX, float *Y, int incY, float c, float s) {
  two_vec_wrap_prep<float>(N, X, incX, Y, incY);
  rot_proc<float>(N, Vec<float>{X, incX}, Vec<float>{Y, incY}, c, s);
}
ORACLE_API void oracle_drot(int N, double *X, int incX, double *Y, int incY, double c, double s) {
  two_vec_wrap_prep<double>(N, X, incX, Y, incY);
  rot_proc<double>(N, Vec<double>{X, incX}, Vec<double>{Y, incY}, c, s);
}
// test/level1/rotm/exo_rotm_wrapper.h:5-44
ORACLE_API void oracle_srotm(int N, float *X, int incX, float *Y, int incY, const float *P) {
  two_vec_wrap_prep<float>(N, X, incX, Y, incY);
  rotm_proc<float>(N, Vec<float>{X, incX}, Vec<float>{Y, incY}, P);
}
ORACLE_API void oracle_drotm(int N, double *X, int incX, double *Y, int incY, const double *P) {
  two_vec_wrap_prep<double>(N, X, incX, Y, incY);
  rotm_proc<double>(N, Vec<double>{X, incX}, Vec<double>{Y, incY}, P);
}

ORACLE_API void oracle_sgemv(int order, int TransA, int M, int N, float alpha, const float *A, int lda, const float *X, int incX, float beta, float *Y, int incY) { gemv_wrap<float>(order, TransA, M, N, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_dgemv(int order, int TransA, int M, int N, double alpha, const double *A, int lda, const double *X, int incX, double beta, double *Y, int incY) { gemv_wrap<double>(order, TransA, M, N, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_sger(int order, int M, int N, float alpha, const float *X, int incX, const float *Y, int incY, float *A, int lda) { ger_wrap<float>(order, M, N, alpha, X, incX, Y, incY, A, lda); }
ORACLE_API void oracle_dger(int order, int M, int N, double alpha, const double *X, int incX, const double *Y, int incY, double *A, int lda) { ger_wrap<double>(order, M, N, alpha, X, incX, Y, incY, A, lda); }
ORACLE_API void oracle_ssymv(int order, int Uplo, int N, float alpha, const float *A, int lda, const float *X, int incX, float beta, float *Y, int incY) { symv_wrap<float>(order, Uplo, N, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_dsymv(int order, int Uplo, int N, double alpha, const double *A, int lda, const double *X, int incX, double beta, double *Y, int incY) { symv_wrap<double>(order, Uplo, N, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_ssyr(int order, int Uplo, int N, float alpha, const float *X, int incX, float *A, int lda) { syr_wrap<float>(order, Uplo, N, alpha, X, incX, A, lda); }
ORACLE_API void oracle_dsyr(int order, int Uplo, int N, double alpha, const double *X, int incX, double *A, int lda) { syr_wrap<double>(order, Uplo, N, alpha, X, incX, A, lda); }
ORACLE_API void oracle_ssyr2(int order, int Uplo, int N, float alpha, const float *X, int incX, const float *Y, int incY, float *A, int lda) { syr2_wrap<float>(order, Uplo, N, alpha, X, incX, Y, incY, A, lda); }
ORACLE_API void oracle_dsyr2(int order, int Uplo, int N, double alpha, const double *X, int incX, const double *Y, int incY, double *A, int lda) { syr2_wrap<double>(order, Uplo, N, alpha, X, incX, Y, incY, A, lda); }
ORACLE_API void oracle_strmv(int order, int Uplo, int TransA, int Diag, int N, const float *A, int lda, float *X, int incX) { trmv_wrap<float>(order, Uplo, TransA, Diag, N, A, lda, X, incX); }
ORACLE_API void oracle_dtrmv(int order, int Uplo, int TransA, int Diag, int N, const double *A, int lda, double *X, int incX) { trmv_wrap<double>(order, Uplo, TransA, Diag, N, A, lda, X, incX); }
ORACLE_API void oracle_strsv(int order, int Uplo, int TransA, int Diag, int N, const float *A, int lda, float *X, int incX) { trsv_wrap<float>(order, Uplo, TransA, Diag, N, A, lda, X, incX); }
ORACLE_API void oracle_dtrsv(int order, int Uplo, int TransA, int Diag, int N, const double *A, int lda, double *X, int incX) { trsv_wrap<double>(order, Uplo, TransA, Diag, N, A, lda, X, incX); }

ORACLE_API void oracle_sgemm(int order, int TransA, int TransB, int M, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc) { gemm_wrap<float>(order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_dgemm(int order, int TransA, int TransB, int M, int N, int K, double alpha, const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc) { gemm_wrap<double>(order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_ssymm(int order, int Side, int Uplo, int M, int N, float alpha, const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc) { symm_wrap<float>(order, Side, Uplo, M, N, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_dsymm(int order, int Side, int Uplo, int M, int N, double alpha, const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc) { symm_wrap<double>(order, Side, Uplo, M, N, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_ssyrk(int order, int Uplo, int Trans, int N, int K, float alpha, const float *A, int lda, float beta, float *C, int ldc) { syrk_wrap<float>(order, Uplo, Trans, N, K, alpha, A, lda, beta, C, ldc); }
ORACLE_API void oracle_dsyrk(int order, int Uplo, int Trans, int N, int K, double alpha, const double *A, int lda, double beta, double *C, int ldc) { syrk_wrap<double>(order, Uplo, Trans, N, K, alpha, A, lda, beta, C, ldc); }

ORACLE_API float oracle_snrm2(int N, const float *X, int incX) { return nrm2_ref<float>(N, X, incX); }
ORACLE_API double oracle_dnrm2(int N, const double *X, int incX) { return nrm2_ref<double>(N, X, incX); }
ORACLE_API long oracle_isamax(int N, const float *X, int incX) { return iamax_ref<float>(N, X, incX); }
ORACLE_API long oracle_idamax(int N, const double *X, int incX) { return iamax_ref<double>(N, X, incX); }
ORACLE_API void oracle_sgbmv(int M, int N, int KL, int KU, float alpha, const float *A, int lda, const float *X, int incX, float beta, float *Y, int incY) { gbmv_wrap<float>(M, N, KL, KU, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_dgbmv(int M, int N, int KL, int KU, double alpha, const double *A, int lda, const double *X, int incX, double beta, double *Y, int incY) { gbmv_wrap<double>(M, N, KL, KU, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_ssbmv(int order, int Uplo, int N, int K, float alpha, const float *A, int lda, const float *X, int incX, float beta, float *Y, int incY) { sbmv_wrap<float>(order, Uplo, N, K, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_dsbmv(int order, int Uplo, int N, int K, double alpha, const double *A, int lda, const double *X, int incX, double beta, double *Y, int incY) { sbmv_wrap<double>(order, Uplo, N, K, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_stbmv(int order, int Uplo, int TransA, int Diag, int N, int K, const float *A, int lda, float *X, int incX) { tb_wrap<float>(false, order, Uplo, TransA, Diag, N, K, A, lda, X, incX); }
ORACLE_API void oracle_dtbmv(int order, int Uplo, int TransA, int Diag, int N, int K, const double *A, int lda, double *X, int incX) { tb_wrap<double>(false, order, Uplo, TransA, Diag, N, K, A, lda, X, incX); }
ORACLE_API void oracle_stbsv(int order, int Uplo, int TransA, int Diag, int N, int K, const float *A, int lda, float *X, int incX) { tb_wrap<float>(true, order, Uplo, TransA, Diag, N, K, A, lda, X, incX); }
ORACLE_API void oracle_dtbsv(int order, int Uplo, int TransA, int Diag, int N, int K, const double *A, int lda, double *X, int incX) { tb_wrap<double>(true, order, Uplo, TransA, Diag, N, K, A, lda, X, incX); }
ORACLE_API void oracle_ssyr2k(int order, int Uplo, int Trans, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc) { syr2k_wrap<float>(order, Uplo, Trans, N, K, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_dsyr2k(int order, int Uplo, int Trans, int N, int K, double alpha, const double *A, int lda, const double *B, int ldb, double beta, double *C, int ldc) { syr2k_wrap<double>(order, Uplo, Trans, N, K, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_strmm(int order, int Side, int Uplo, int TransA, int Diag, int M, int N, float alpha, const float *A, int lda, float *B, int ldb) { trmm_wrap<float>(order, Side, Uplo, TransA, Diag, M, N, alpha, A, lda, B, ldb); }
ORACLE_API void oracle_dtrmm(int order, int Side, int Uplo, int TransA, int Diag, int M, int N, double alpha, const double *A, int lda, double *B, int ldb) { trmm_wrap<double>(order, Side, Uplo, TransA, Diag, M, N, alpha, A, lda, B, ldb); }

// ----- the same restatements in double-word arithmetic (T = Dw)
// Arguments as oracle_d<op>; every array is a Dw array (pairs {hi, lo} of
// doubles, inputs entered as {x, 0}), scalars are doubles, and returned
// scalars are rounded to double.  These are the d-precision references.

ORACLE_API double oracle_dw_dasum(int N, const Dw *X, int incX) { return asum_wrap<Dw>(N, X, incX).value(); }
ORACLE_API void oracle_dw_daxpy(int N, double alpha, const Dw *X, int incX, Dw *Y, int incY) { axpy_wrap<Dw>(N, alpha, X, incX, Y, incY); }
ORACLE_API double oracle_dw_ddot(int N, const Dw *X, int incX, const Dw *Y, int incY) { return dot_wrap<Dw>(N, X, incX, Y, incY).value(); }
ORACLE_API void oracle_dw_dscal(int N, double alpha, Dw *X, int incX) { scal_wrap<Dw>(N, alpha, X, incX); }
ORACLE_API void oracle_dw_drot(int N, Dw *X, int incX, Dw *Y, int incY, double c, double s) {
  two_vec_wrap_prep<Dw>(N, X, incX, Y, incY);
  rot_proc<Dw>(N, Vec<Dw>{X, incX}, Vec<Dw>{Y, incY}, c, s);
}
ORACLE_API void oracle_dw_drotm(int N, Dw *X, int incX, Dw *Y, int incY, const Dw *P) {
  two_vec_wrap_prep<Dw>(N, X, incX, Y, incY);
  rotm_proc<Dw>(N, Vec<Dw>{X, incX}, Vec<Dw>{Y, incY}, P);
}
ORACLE_API void oracle_dw_dgemv(int order, int TransA, int M, int N, double alpha, const Dw *A, int lda, const Dw *X, int incX, double beta, Dw *Y, int incY) { gemv_wrap<Dw>(order, TransA, M, N, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_dw_dger(int order, int M, int N, double alpha, const Dw *X, int incX, const Dw *Y, int incY, Dw *A, int lda) { ger_wrap<Dw>(order, M, N, alpha, X, incX, Y, incY, A, lda); }
ORACLE_API void oracle_dw_dsymv(int order, int Uplo, int N, double alpha, const Dw *A, int lda, const Dw *X, int incX, double beta, Dw *Y, int incY) { symv_wrap<Dw>(order, Uplo, N, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_dw_dsyr(int order, int Uplo, int N, double alpha, const Dw *X, int incX, Dw *A, int lda) { syr_wrap<Dw>(order, Uplo, N, alpha, X, incX, A, lda); }
ORACLE_API void oracle_dw_dsyr2(int order, int Uplo, int N, double alpha, const Dw *X, int incX, const Dw *Y, int incY, Dw *A, int lda) { syr2_wrap<Dw>(order, Uplo, N, alpha, X, incX, Y, incY, A, lda); }
ORACLE_API void oracle_dw_dtrmv(int order, int Uplo, int TransA, int Diag, int N, const Dw *A, int lda, Dw *X, int incX) { trmv_wrap<Dw>(order, Uplo, TransA, Diag, N, A, lda, X, incX); }
ORACLE_API void oracle_dw_dtrsv(int order, int Uplo, int TransA, int Diag, int N, const Dw *A, int lda, Dw *X, int incX) { trsv_wrap<Dw>(order, Uplo, TransA, Diag, N, A, lda, X, incX); }
ORACLE_API void oracle_dw_dgemm(int order, int TransA, int TransB, int M, int N, int K, double alpha, const Dw *A, int lda, const Dw *B, int ldb, double beta, Dw *C, int ldc) { gemm_wrap<Dw>(order, TransA, TransB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_dw_dsymm(int order, int Side, int Uplo, int M, int N, double alpha, const Dw *A, int lda, const Dw *B, int ldb, double beta, Dw *C, int ldc) { symm_wrap<Dw>(order, Side, Uplo, M, N, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_dw_dsyrk(int order, int Uplo, int Trans, int N, int K, double alpha, const Dw *A, int lda, double beta, Dw *C, int ldc) { syrk_wrap<Dw>(order, Uplo, Trans, N, K, alpha, A, lda, beta, C, ldc); }
ORACLE_API void oracle_dw_dgbmv(int M, int N, int KL, int KU, double alpha, const Dw *A, int lda, const Dw *X, int incX, double beta, Dw *Y, int incY) { gbmv_wrap<Dw>(M, N, KL, KU, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_dw_dsbmv(int order, int Uplo, int N, int K, double alpha, const Dw *A, int lda, const Dw *X, int incX, double beta, Dw *Y, int incY) { sbmv_wrap<Dw>(order, Uplo, N, K, alpha, A, lda, X, incX, beta, Y, incY); }
ORACLE_API void oracle_dw_dtbmv(int order, int Uplo, int TransA, int Diag, int N, int K, const Dw *A, int lda, Dw *X, int incX) { tb_wrap<Dw>(false, order, Uplo, TransA, Diag, N, K, A, lda, X, incX); }
ORACLE_API void oracle_dw_dtbsv(int order, int Uplo, int TransA, int Diag, int N, int K, const Dw *A, int lda, Dw *X, int incX) { tb_wrap<Dw>(true, order, Uplo, TransA, Diag, N, K, A, lda, X, incX); }
ORACLE_API void oracle_dw_dsyr2k(int order, int Uplo, int Trans, int N, int K, double alpha, const Dw *A, int lda, const Dw *B, int ldb, double beta, Dw *C, int ldc) { syr2k_wrap<Dw>(order, Uplo, Trans, N, K, alpha, A, lda, B, ldb, beta, C, ldc); }
ORACLE_API void oracle_dw_dtrmm(int order, int Side, int Uplo, int TransA, int Diag, int M, int N, double alpha, const Dw *A, int lda, Dw *B, int ldb) { trmm_wrap<Dw>(order, Side, Uplo, TransA, Diag, M, N, alpha, A, lda, B, ldb); }

// nrm2 with the same scaling as nrm2_ref, the sum of squares in double-word
// and a double-word square root (one Newton correction of sqrt(hi)).
ORACLE_API double oracle_dw_dnrm2(int N, const Dw *X, int incX) {
  g_status = 0;
  if (N < 1) return 0.0;
  if (incX < 0) X = X + long(1 - N) * incX;
  double scale = 0;
  bool nan = false;
  for (long i = 0; i < N; ++i) {
    const double v = std::fabs(X[i * incX].hi);
    if (v != v) nan = true;
    if (v > scale) scale = v;
  }
  if (nan) return NAN;
  if (scale == 0 || std::isinf(scale)) return scale;
  Dw ss(0.0);
  for (long i = 0; i < N; ++i) {
    const Dw v = X[i * incX] / Dw(scale);
    ss += v * v;
  }
  const double s0 = std::sqrt(ss.hi);
  const Dw root = Dw(s0) + (ss - Dw(s0) * Dw(s0)) / Dw(2.0 * s0);
  return (Dw(scale) * root).value();
}

// ----- double-double high-precision references (results rounded to double)

// Dot2 over strided windows (pointers already rebased by the caller).
ORACLE_API double oracle_dd_dot(long n, const double *x, long incx, const double *y, long incy) {
  DD acc{0.0, 0.0};
  for (long i = 0; i < n; ++i) dd_add_prod(acc, x[i * incx], y[i * incy]);
  DD r = dd_norm(acc);
  return r.hi + r.lo;
}

// y_out[i] = alpha * sum_j op(A)[i,j] x[j] + beta * y_in[i] in double-double;
// trans != 0 means op(A) = A^T.  m x n is the shape of op(A); A is row-major.
ORACLE_API void oracle_dd_gemv(int trans, long m, long n, double alpha, const double *A, long lda, const double *x, double beta, const double *y_in, double *y_out) {
  for (long i = 0; i < m; ++i) {
    DD acc{0.0, 0.0};
    for (long j = 0; j < n; ++j) dd_add_prod(acc, trans ? A[j * lda + i] : A[i * lda + j], x[j]);
    DD r = dd_norm(acc);
    // alpha * (hi + lo) + beta * y, each product exact-split then summed
    DD out{0.0, 0.0};
    dd_add_prod(out, alpha, r.hi);
    dd_add_prod(out, alpha, r.lo);
    dd_add_prod(out, beta, y_in[i]);
    out = dd_norm(out);
    y_out[i] = out.hi + out.lo;
  }
}

// Forward/back substitution in double-double.  x holds b on entry (unit
// stride) and the double-rounded solution on exit; x_lo receives the low
// parts so callers can measure forward error below one ulp.
ORACLE_API void oracle_dd_trsv(int uplo, int trans, int diag, long n, const double *A, long lda, double *x, double *x_lo) {
  std::vector<DD> xs(n);
  for (long i = 0; i < n; ++i) xs[i] = DD{x[i], 0.0};
  auto at = [&](long r, long c) { return trans ? A[c * lda + r] : A[r * lda + c]; };
  const bool lower_eff = (uplo == kLower) != (trans != 0);
  for (long t = 0; t < n; ++t) {
    const long i = lower_eff ? t : n - 1 - t;
    DD acc{xs[i].hi, xs[i].lo};
    const long j0 = lower_eff ? 0 : i + 1, j1 = lower_eff ? i : n;
    for (long j = j0; j < j1; ++j) {
      const double aij = at(i, j);
      dd_add_prod(acc, -aij, xs[j].hi);
      dd_add_prod(acc, -aij, xs[j].lo);
    }
    acc = dd_norm(acc);
    if (diag == kNonUnit) {
      // double-double divide by a double: q1 = hi/d, r = acc - q1*d, q2 = r/d
      const double d = at(i, i);
      double q1 = acc.hi / d;
      double p, pe;
      two_prod(q1, d, p, pe);
      double r = ((acc.hi - p) - pe) + acc.lo;
      double q2 = r / d;
      double s, e;
      two_sum(q1, q2, s, e);
      acc = DD{s, e};
    }
    xs[i] = acc;
  }
  for (long i = 0; i < n; ++i) {
    x[i] = xs[i].hi + xs[i].lo;
    if (x_lo) x_lo[i] = (xs[i].hi - x[i]) + xs[i].lo;
  }
}

// Selected entries of alpha * op(A) op(B) + beta * C in double-double:
// out[t] for (rows[t], cols[t]), t < count.  op(A) is m x k, op(B) is k x n.
ORACLE_API void oracle_dd_gemm_entries(int transa, int transb, long k, double alpha, const double *A, long lda, const double *B, long ldb, double beta, const double *C, long ldc, const long *rows, const long *cols, long count, double *out) {
  for (long t = 0; t < count; ++t) {
    const long i = rows[t], j = cols[t];
    DD acc{0.0, 0.0};
    for (long p = 0; p < k; ++p) {
      const double a = transa ? A[p * lda + i] : A[i * lda + p];
      const double b = transb ? B[j * ldb + p] : B[p * ldb + j];
      dd_add_prod(acc, a, b);
    }
    DD r = dd_norm(acc);
    DD o{0.0, 0.0};
    dd_add_prod(o, alpha, r.hi);
    dd_add_prod(o, alpha, r.lo);
    if (C) dd_add_prod(o, beta, C[i * ldc + j]);
    o = dd_norm(o);
    out[t] = o.hi + o.lo;
  }
}

// ----- multi-threaded drivers of the same algorithms (CPU baseline timing)

ORACLE_API void oracle_par_saxpy(int nthreads, int N, float alpha, const float *X, float *Y) {
  parallel_for(nthreads, N, [&](int, long lo, long hi) { oracle_saxpy((int)(hi - lo), alpha, X + lo, 1, Y + lo, 1); });
}
ORACLE_API void oracle_par_daxpy(int nthreads, int N, double alpha, const double *X, double *Y) {
  parallel_for(nthreads, N, [&](int, long lo, long hi) { oracle_daxpy((int)(hi - lo), alpha, X + lo, 1, Y + lo, 1); });
}
ORACLE_API float oracle_par_sdot(int nthreads, int N, const float *X, const float *Y) {
  std::vector<float> part(nthreads > 0 ? nthreads : 1, 0.0f);
  parallel_for(nthreads, N, [&](int t, long lo, long hi) { part[t] = oracle_sdot((int)(hi - lo), X + lo, 1, Y + lo, 1); });
  float r = 0.0f;
  for (float p : part) r += p;
  return r;
}
ORACLE_API double oracle_par_ddot(int nthreads, int N, const double *X, const double *Y) {
  std::vector<double> part(nthreads > 0 ? nthreads : 1, 0.0);
  parallel_for(nthreads, N, [&](int t, long lo, long hi) { part[t] = oracle_ddot((int)(hi - lo), X + lo, 1, Y + lo, 1); });
  double r = 0.0;
  for (double p : part) r += p;
  return r;
}
ORACLE_API double oracle_par_dsdot(int nthreads, int N, const float *X, const float *Y) {
  std::vector<double> part(nthreads > 0 ? nthreads : 1, 0.0);
  parallel_for(nthreads, N, [&](int t, long lo, long hi) { part[t] = oracle_dsdot((int)(hi - lo), X + lo, 1, Y + lo, 1); });
  double r = 0.0;
  for (double p : part) r += p;
  return r;
}
// y = beta*y + alpha*op(A) x with rows (NoTrans) or columns (Trans) of y split
ORACLE_API void oracle_par_sgemv(int nthreads, int TransA, int M, int N, float alpha, const float *A, int lda, const float *X, float beta, float *Y) {
  const long ylen = TransA == kNoTrans ? M : N;
  parallel_for(nthreads, ylen, [&](int, long lo, long hi) {
    if (TransA == kNoTrans)
      oracle_sgemv(kRowMajor, kNoTrans, (int)(hi - lo), N, alpha, A + lo * lda, lda, X, 1, beta, Y + lo, 1);
    else
      oracle_sgemv(kRowMajor, TransA, M, (int)(hi - lo), alpha, A + lo, lda, X, 1, beta, Y + lo, 1);
  });
}
// Blocked lower/no-trans solve: the off-diagonal panel of each 256-row block is
// a parallel row-dot over the already solved prefix (trsv.py:31-36 per row),
// the 256 x 256 diagonal block runs the proc sequentially.
ORACLE_API void oracle_par_dtrsv_lnn(int nthreads, int N, const double *A, int lda, double *X) {
  const long B = 256;
  for (long k0 = 0; k0 < N; k0 += B) {
    const long k1 = k0 + B < N ? k0 + B : N;
    parallel_for(nthreads, k1 - k0, [&](int, long lo, long hi) {
      for (long i = k0 + lo; i < k0 + hi; ++i) {
        double dot = 0.0;
        const double *ai = A + i * lda;
        for (long j = 0; j < k0; ++j) dot += ai[j] * X[j];
        X[i] -= dot;
      }
    });
    oracle_dtrsv(kRowMajor, kLower, kNoTrans, kNonUnit, (int)(k1 - k0), A + k0 * lda + k0, lda, X + k0, 1);
  }
}
ORACLE_API void oracle_par_sgemm(int nthreads, int TransA, int TransB, int M, int N, int K, float alpha, const float *A, int lda, const float *B, int ldb, float beta, float *C, int ldc) {
  Mat<float> a{const_cast<float *>(A), lda}, b{const_cast<float *>(B), ldb}, c{C, ldc};
  parallel_for(nthreads, M, [&](int, long lo, long hi) {
    mscal_proc<float>(hi - lo, N, beta, Mat<float>{C + lo * ldc, ldc});
    gemm_rows<float>(TransA, TransB, lo, hi, N, K, alpha, a, b, c);
  });
}
