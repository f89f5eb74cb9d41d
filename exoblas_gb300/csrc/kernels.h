// Launchers for the device kernels.  All pointers are device pointers; vector
// element i lives at p[i * inc] (inc may be negative, the pointer already
// rebased to element 0 exactly as the reference wrappers do).  Launchers
// enqueue on ctx().stream and never synchronise.
#pragma once

#include "common.cuh"

namespace exb {

namespace l1 {
template <typename T>
void axpy(long n, T alpha, const T *x, long incx, T *y, long incy);
template <typename T>
void scal(long n, T alpha, T *x, long incx);  // alpha == 0 writes zeros
template <typename T>
void copy(long n, const T *x, long incx, T *y, long incy);
template <typename T>
void swap(long n, T *x, long incx, T *y, long incy);
template <typename T>
void rot(long n, T *x, long incx, T *y, long incy, T c, T s);
// P[0] is the flag (-1, 0, 1 act; anything else is a no-op); P on the host
template <typename T>
void rotm(long n, T *x, long incx, T *y, long incy, const T P[5]);
template <typename T>
void asum(long n, const T *x, long incx, T *result);
template <typename T>
void dot(long n, const T *x, long incx, const T *y, long incy, T *result);
// result (double) = sum of double(x_i) * double(y_i); if sresult != nullptr
// also writes float(result + sb) there (sdsdot)
void dsdot(long n, const float *x, long incx, const float *y, long incy, double *result, float sb, float *sresult);
// sqrt(sum x_i^2) without overflow or underflow; 0-based index of the first
// largest |x_i| (device results)
template <typename T>
void nrm2(long n, const T *x, long incx, T *result);
template <typename T>
void iamax(long n, const T *x, long incx, size_t *result);
// dasum with integer significand sums on the bit patterns (level1_ext.cu)
void dasum_words(long n, const double *x, long incx, double *result);
}  // namespace l1

namespace l2 {
// y = beta*y + alpha*op(A) x; A row-major rows x cols (the caller's M x N)
template <typename T>
void gemv(bool trans, long rows, long cols, T alpha, const T *A, long lda, const T *x, long incx, T beta, T *y,
          long incy);
template <typename T>
void ger(long m, long n, T alpha, const T *x, long incx, const T *y, long incy, T *A, long lda);
template <typename T>
void symv(bool upper, long n, T alpha, const T *A, long lda, const T *x, long incx, T beta, T *y, long incy);
template <typename T>
void syr(bool upper, long n, T alpha, const T *x, long incx, T *A, long lda);
template <typename T>
void syr2(bool upper, long n, T alpha, const T *x, long incx, const T *y, long incy, T *A, long lda);
template <typename T>
void trmv(bool upper, bool trans, bool unit, long n, const T *A, long lda, T *x, long incx);
template <typename T>
void trsv(bool upper, bool trans, bool unit, long n, const T *A, long lda, T *x, long incx);
// banded (row-major CBLAS band storage)
template <typename T>
void gbmv(long m, long n, long kl, long ku, T alpha, const T *A, long lda, const T *x, long incx, T beta, T *y,
          long incy);
template <typename T>
void sbmv(bool upper, long n, long k, T alpha, const T *A, long lda, const T *x, long incx, T beta, T *y, long incy);
template <typename T>
void tbmv(bool upper, bool trans, bool unit, long n, long k, const T *A, long lda, T *x, long incx);
template <typename T>
void tbsv(bool upper, bool trans, bool unit, long n, long k, const T *A, long lda, T *x, long incx);
}  // namespace l2

namespace l3 {
// CUDA-core (FFMA / DFMA) paths
template <typename T>
void gemm_simt(bool ta, bool tb, long m, long n, long k, T alpha, const T *A, long lda, const T *B, long ldb, T beta,
               T *C, long ldc);
template <typename T>
void symm_simt(bool left, bool upper, long m, long n, T alpha, const T *A, long lda, const T *B, long ldb, T beta,
               T *C, long ldc);
template <typename T>
void syrk_simt(bool upper, bool trans, long n, long k, T alpha, const T *A, long lda, T beta, T *C, long ldc);
template <typename T>
void syr2k_simt(bool upper, bool trans, long n, long k, T alpha, const T *A, long lda, const T *B, long ldb, T beta,
                T *C, long ldc);
template <typename T>
void trmm_simt(bool left, bool upper, bool trans, bool unit, long m, long n, T alpha, const T *A, long lda, T *B,
               long ldb);
// tcgen05 tensor-core paths: FP32 through three BF16 terms per operand
void gemm_split_bf16(bool ta, bool tb, long m, long n, long k, float alpha, const float *A, long lda, const float *B,
                     long ldb, float beta, float *C, long ldc);
void symm_split_bf16(bool left, bool upper, long m, long n, float alpha, const float *A, long lda, const float *B,
                     long ldb, float beta, float *C, long ldc);
void syrk_split_bf16(bool upper, bool trans, long n, long k, float alpha, const float *A, long lda, float beta,
                     float *C, long ldc);
void syr2k_split_bf16(bool upper, bool trans, long n, long k, float alpha, const float *A, long lda, const float *B,
                      long ldb, float beta, float *C, long ldc);
// tcgen05 Ozaki slice emulation of dgemm; false when an input is not finite
// (nothing written; the caller uses the FP64 FMA kernel)
bool dgemm_ozaki(bool ta, bool tb, long m, long n, long k, double alpha, const double *A, long lda, const double *B,
                 long ldb, double beta, double *C, long ldc);
bool dsymm_ozaki(bool left, bool upper, long m, long n, double alpha, const double *A, long lda, const double *B,
                 long ldb, double beta, double *C, long ldc);
bool dsyrk_ozaki(bool upper, bool trans, long n, long k, double alpha, const double *A, long lda, double beta,
                 double *C, long ldc);
bool dsyr2k_ozaki(bool upper, bool trans, long n, long k, double alpha, const double *A, long lda, const double *B,
                  long ldb, double beta, double *C, long ldc);
// A group of independent FP32 products C_g = alpha_g op(A_g) op(B_g) +
// beta_g C_g on the split-BF16 tensor-core path (gemm_tc.cu): built once
// (slice planes, tensor maps, tile items on the device), launched as one
// grouped split and one grouped persistent product on a stream.  Each
// product's result equals gemm_split_bf16 of the same call bit for bit.
struct TcGroupOp {
  bool ta, tb;
  int m, n, k;
  float alpha, beta;
  const float *A;
  long lda;
  const float *B;
  long ldb;
  float *C;
  long ldc;
};
struct TcGroup;
TcGroup *tc_group_create(const TcGroupOp *ops, int n);
int tc_group_launch(const TcGroup *g, cudaStream_t s);  // returns the kernels launched
void tc_group_destroy(TcGroup *g);

}  // namespace l3

}  // namespace exb
