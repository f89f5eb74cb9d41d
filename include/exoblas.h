/*
 * exoblas.h - C ABI of libexoblas_gb300.so, a GB300 (sm_103a) implementation
 * of the ExoBLAS dense BLAS hot path.
 *
 * Every exo_<p><op> entry point keeps the signature, the CBLAS argument
 * order, the flag values and the special cases of the ExoBLAS wrapper it
 * replaces (cited beside each declaration as reference file:line).  Those
 * wrappers are the C++ headers test/level{1,2,3}/<op>/exo_<op>_wrapper.h of
 * exo-lang/ExoBLAS; they dispatch to Exo-generated CPU procs.  Here the same
 * calls run hand-written CUDA kernels on the current CUDA device.
 *
 * Pointers may be host memory (pageable or pinned) or device memory
 * (cudaMalloc / managed); the library asks the CUDA driver which one each
 * pointer is.  Host operands are staged through device memory and copied
 * back; device operands are used in place.  By default every call returns
 * only after its results are visible to the caller (CBLAS semantics); see
 * exoblas_set_blocking for the asynchronous device-pointer mode.
 *
 * Errors: the reference wrappers throw a C++ exception when Order is not
 * CblasRowMajor (e.g. test/level3/gemm/exo_gemm_wrapper.h:15-17).  This
 * library never throws across the ABI: it leaves every output untouched,
 * records a status for the calling thread (exoblas_get_status) and, if one
 * is installed, calls the error handler (exoblas_set_error_handler).
 */
#ifndef EXOBLAS_GB300_H
#define EXOBLAS_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define EXOBLAS_API __attribute__((visibility("default")))
#else
#define EXOBLAS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* CBLAS flag values, identical to test/common/cblas.h:10-18 of the reference
 * (and to every netlib-compatible cblas.h, whose definitions are used when
 * that header was included first). */
#ifndef CBLAS_H
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
enum CBLAS_UPLO { CblasUpper = 121, CblasLower = 122 };
enum CBLAS_DIAG { CblasNonUnit = 131, CblasUnit = 132 };
enum CBLAS_SIDE { CblasLeft = 141, CblasRight = 142 };
#endif

/* ------------------------------------------------------------ status --- */
enum EXOBLAS_STATUS {
  EXOBLAS_SUCCESS = 0,
  EXOBLAS_UNSUPPORTED_ORDER = 1, /* Order != CblasRowMajor (the reference throws) */
  EXOBLAS_INVALID_VALUE = 2,     /* bad flag, negative size, lda too small, zero output stride */
  EXOBLAS_CUDA_ERROR = 3,        /* a CUDA runtime call failed */
  EXOBLAS_ALLOC_FAILED = 4,      /* device workspace or staging allocation failed */
  EXOBLAS_TIMEOUT = 5,           /* a kernel's bounded wait ran out; outputs are undefined */
  EXOBLAS_NOT_SUPPORTED = 6      /* requested mode not available on this device */
};

/* Status of the last exo_* / exoblas_* call made by the calling thread. */
EXOBLAS_API int exoblas_get_status(void);
EXOBLAS_API const char *exoblas_status_string(int status);
/* Called (on the calling thread) whenever a call fails; NULL removes it. */
typedef void (*exoblas_error_handler)(int status, const char *function, const char *message);
EXOBLAS_API void exoblas_set_error_handler(exoblas_error_handler handler);

/* ------------------------------------------------------ execution state - */
/* Stream used by the calling thread's subsequent calls on the current device
 * (a cudaStream_t, including cudaStreamLegacy / cudaStreamPerThread; NULL
 * selects the library's own non-blocking stream, which is not ordered with
 * the legacy default stream).
 * Work already queued by this thread on its previous stream is synchronised
 * first, so scratch memory is never shared by two streams at once. */
EXOBLAS_API int exoblas_set_stream(void *stream);
EXOBLAS_API void *exoblas_get_stream(void);
/* blocking = 1 (default): calls return once results are visible on the host.
 * blocking = 0: calls whose operands are ALL device pointers return after
 * queuing their kernels on the thread's stream; scalar-returning reductions
 * (asum, dot, dsdot, sdsdot) still wait for their result.  Use the
 * exoblas_*_device variants below for fully asynchronous reductions. */
EXOBLAS_API int exoblas_set_blocking(int blocking);
/* Waits for the thread's queued work.  Also reports EXOBLAS_TIMEOUT when a
 * kernel queued in non-blocking mode (trsv) gave up a bounded wait. */
EXOBLAS_API int exoblas_synchronize(void);
/* Self-test of the bounded-wait path (no reference counterpart): launches one
 * kernel that waits on a device flag nothing sets, gives up after `seconds`
 * (0 < seconds <= 1), records the expiry in the device status word and
 * returns.  The call then reports EXOBLAS_TIMEOUT through the same path as
 * the solvers' bounded waits; the thread's context stays usable. */
EXOBLAS_API int exoblas_selftest_wait_timeout(double seconds);

/* Arithmetic used by exo_sgemm/ssymm/ssyrk/ssyr2k and exo_dgemm/dsymm/dsyrk/dsyr2k:
 *   EXOBLAS_PRECISION_NATIVE    FP32 FFMA / FP64 DFMA kernels (default)
 *   EXOBLAS_PRECISION_SPLIT_BF16 sgemm/ssymm/ssyrk/ssyr2k: each FP32 operand split
 *                               into three BF16 terms, products on tcgen05
 *                               tensor cores, FP32 accumulation
 *   EXOBLAS_PRECISION_OZAKI     dgemm/dsymm/dsyrk/dsyr2k: Ozaki slice emulation
 *                               with exact integer accumulation of
 *                               small-integer slices (inputs holding NaN or
 *                               infinity take the DFMA kernels)
 * The environment variable EXOBLAS_PRECISION_MODE (native | split_bf16 |
 * ozaki) sets the initial value for every thread. */
enum EXOBLAS_PRECISION { EXOBLAS_PRECISION_NATIVE = 0, EXOBLAS_PRECISION_SPLIT_BF16 = 1, EXOBLAS_PRECISION_OZAKI = 2 };
EXOBLAS_API int exoblas_set_precision(int mode);
EXOBLAS_API int exoblas_get_precision(void);

/* Column-major calls (CblasColMajor) for this thread: rejected by default,
 * as the reference rejects them; when enabled every exo_* entry point with
 * an Order argument computes the column-major (CBLAS) result by running the
 * row-major call on the transposed view of its operands.  The environment
 * variable EXOBLAS_COLUMN_MAJOR=1 enables it for every thread. */
EXOBLAS_API int exoblas_set_column_major(int enable);
EXOBLAS_API int exoblas_get_column_major(void);

/* Number of CUDA kernels this library has launched in the calling process. */
EXOBLAS_API unsigned long long exoblas_kernel_launches(void);
/* Bytes this process has copied host->device and device->host while staging
 * host operands (no counterpart in the reference, which has no device). */
EXOBLAS_API void exoblas_staged_bytes(unsigned long long *h2d, unsigned long long *d2h);

/* ------------------------------------------------------------ level 1 --- */
/* test/level1/asum/exo_asum_wrapper.h:5-23 (incX < 0 returns 0) */
EXOBLAS_API float exo_sasum(const int N, const float *X, const int incX);
EXOBLAS_API double exo_dasum(const int N, const double *X, const int incX);
/* nrm2 and i?amax: standard level-1 routines the reference lacks
 * (README.md:15), with reference BLAS semantics.  nrm2: free of overflow and
 * underflow, 0 for N < 1, any increment (negative walks the vector
 * backwards, 0 repeats X[0]); i?amax: 0 for N < 1 or incX < 1, else the
 * 0-based index (as cblas_i?amax) of the first element of largest magnitude */
EXOBLAS_API float exo_snrm2(const int N, const float *X, const int incX);
EXOBLAS_API double exo_dnrm2(const int N, const double *X, const int incX);
EXOBLAS_API size_t exo_isamax(const int N, const float *X, const int incX);
EXOBLAS_API size_t exo_idamax(const int N, const double *X, const int incX);
/* test/level1/axpy/exo_axpy_wrapper.h:5-34 (alpha == 0 returns) */
EXOBLAS_API void exo_saxpy(const int N, const float alpha, const float *X, const int incX, float *Y, const int incY);
EXOBLAS_API void exo_daxpy(const int N, const double alpha, const double *X, const int incX, double *Y, const int incY);
/* test/level1/dot/exo_dot_wrapper.h:5-27 */
EXOBLAS_API float exo_sdot(const int N, const float *X, const int incX, const float *Y, const int incY);
EXOBLAS_API double exo_ddot(const int N, const double *X, const int incX, const double *Y, const int incY);
/* test/level1/dsdot/exo_dsdot_wrapper.h:5-25 */
EXOBLAS_API double exo_dsdot(const int N, const float *X, const int incX, const float *Y, const int incY);
/* test/level1/sdsdot/exo_sdsdot.h:5-26 */
EXOBLAS_API float exo_sdsdot(const int N, const float alpha, const float *X, const int incX, const float *Y, const int incY);
/* test/level1/copy/exo_copy_wrapper.h:5-23 */
EXOBLAS_API void exo_scopy(const int N, const float *X, const int incX, float *Y, const int incY);
EXOBLAS_API void exo_dcopy(const int N, const double *X, const int incX, double *Y, const int incY);
/* test/level1/swap/exo_swap_wrapper.h:5-23 */
EXOBLAS_API void exo_sswap(const int N, float *X, const int incX, float *Y, const int incY);
EXOBLAS_API void exo_dswap(const int N, double *X, const int incX, double *Y, const int incY);
/* test/level1/scal/exo_scal_wrapper.h:7-35 (alpha == 1 and incX < 0 return) */
EXOBLAS_API void exo_sscal(const int N, const float alpha, float *X, const int incX);
EXOBLAS_API void exo_dscal(const int N, const double alpha, double *X, const int incX);
/* test/level1/rot/exo_rot_wrapper.h:5-23 */
EXOBLAS_API void exo_srot(const int N, float *X, const int incX, float *Y, const int incY, const float c, const float s);
EXOBLAS_API void exo_drot(const int N, double *X, const int incX, double *Y, const int incY, const double c, const double s);
/* test/level1/rotm/exo_rotm_wrapper.h:5-44 (P[0] not in {-1, 0, 1}: no-op) */
EXOBLAS_API void exo_srotm(const int N, float *X, const int incX, float *Y, const int incY, const float *P);
EXOBLAS_API void exo_drotm(const int N, double *X, const int incX, double *Y, const int incY, const double *P);

/* Device-result reductions (no counterpart in the reference: the reference
 * returns the scalar).  All pointers must be device pointers; *result is
 * written by a kernel on the thread's stream and the call does not wait. */
EXOBLAS_API int exoblas_sasum_device(const int N, const float *X, const int incX, float *result);
EXOBLAS_API int exoblas_dasum_device(const int N, const double *X, const int incX, double *result);
EXOBLAS_API int exoblas_sdot_device(const int N, const float *X, const int incX, const float *Y, const int incY, float *result);
EXOBLAS_API int exoblas_ddot_device(const int N, const double *X, const int incX, const double *Y, const int incY, double *result);
EXOBLAS_API int exoblas_dsdot_device(const int N, const float *X, const int incX, const float *Y, const int incY, double *result);
/* device-result nrm2 / i?amax (same semantics as exo_?nrm2 / exo_i?amax) */
EXOBLAS_API int exoblas_snrm2_device(const int N, const float *X, const int incX, float *result);
EXOBLAS_API int exoblas_dnrm2_device(const int N, const double *X, const int incX, double *result);
EXOBLAS_API int exoblas_isamax_device(const int N, const float *X, const int incX, size_t *result);
EXOBLAS_API int exoblas_idamax_device(const int N, const double *X, const int incX, size_t *result);

/* ------------------------------------------------------------ level 2 --- */
/* test/level2/gemv/exo_gemv_wrapper.h:7-39 */
EXOBLAS_API void exo_sgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE TransA, const int M, const int N, const float alpha,
               const float *A, const int lda, const float *X, const int incX, const float beta, float *Y, const int incY);
EXOBLAS_API void exo_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE TransA, const int M, const int N, const double alpha,
               const double *A, const int lda, const double *X, const int incX, const double beta, double *Y, const int incY);
/* test/level2/ger/exo_ger_wrapper.h:7-34 (Order is not checked; alpha == 0 returns) */
EXOBLAS_API void exo_sger(const enum CBLAS_ORDER order, const int M, const int N, const float alpha, const float *X, const int incX,
              const float *Y, const int incY, float *A, const int lda);
EXOBLAS_API void exo_dger(const enum CBLAS_ORDER order, const int M, const int N, const double alpha, const double *X, const int incX,
              const double *Y, const int incY, double *A, const int lda);
/* test/level2/symv/exo_symv_wrapper.h:7-34 */
EXOBLAS_API void exo_ssymv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const float alpha, const float *A,
               const int lda, const float *X, const int incX, const float beta, float *Y, const int incY);
EXOBLAS_API void exo_dsymv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const double alpha, const double *A,
               const int lda, const double *X, const int incX, const double beta, double *Y, const int incY);
/* test/level2/syr/exo_syr_wrapper.h:5-32 (alpha == 0 returns) */
EXOBLAS_API void exo_ssyr(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const float alpha, const float *X,
              const int incX, float *A, const int lda);
EXOBLAS_API void exo_dsyr(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const double alpha, const double *X,
              const int incX, double *A, const int lda);
/* test/level2/syr2/exo_syr2_wrapper.h:5-36 (Order is not checked; alpha == 0 returns) */
EXOBLAS_API void exo_ssyr2(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const float alpha, const float *X,
               const int incX, const float *Y, const int incY, float *A, const int lda);
EXOBLAS_API void exo_dsyr2(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const double alpha, const double *X,
               const int incX, const double *Y, const int incY, double *A, const int lda);
/* test/level2/trmv/exo_trmv_wrapper.h:7-29 */
EXOBLAS_API void exo_strmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const float *A, const int lda, float *X, const int incX);
EXOBLAS_API void exo_dtrmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const double *A, const int lda, double *X, const int incX);
/* test/level2/trsv/exo_trsv_wrapper.h:7-29 */
EXOBLAS_API void exo_strsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const float *A, const int lda, float *X, const int incX);
EXOBLAS_API void exo_dtrsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const double *A, const int lda, double *X, const int incX);

/* exoblas_sgemv_noalloc: no counterpart in the reference.  exo_sgemv for
 * callers that cannot allocate device memory (e.g. a plugin inside a
 * framework whose allocator owns all device memory, or a loop that must not
 * block in the driver's allocator).  Same arguments and arithmetic as
 * exo_sgemv plus a cudaStream_t (NULL: the legacy default stream), and
 * column-major calls are accepted exactly when exo_sgemv accepts them
 * (exoblas_set_column_major); A, X and Y must be device pointers on the
 * current device.  The call queues its kernels and returns without
 * waiting, and returns the status (also readable with exoblas_get_status).
 * It allocates nothing: its scratch is a fixed 4 MiB array inside the
 * library, held on every GPU that loads it.  Limit: a Trans call needs
 * 4*N bytes (one column-sum chunk) plus, when X is strided or not 16-byte
 * aligned, 4*M bytes for a packed copy of X; a NoTrans call with such an X
 * needs 4*N bytes; larger problems are rejected with EXOBLAS_INVALID_VALUE
 * before any work is queued.  A Trans call whose packed X leaves room for
 * fewer column-sum chunks than exo_sgemv would use runs with fewer chunks,
 * so its sums run in another order and can differ from exo_sgemv's in the
 * last bits (both stay within the same error bound).  Every call shares the array, so calls that
 * overlap on the GPU race and must be serialised.  The first call on each
 * device looks the array's address up (cudaGetSymbolAddress); make it before
 * any stream capture starts on that device. */
EXOBLAS_API int exoblas_sgemv_noalloc(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE TransA, const int M,
                                      const int N, const float alpha, const float *A, const int lda, const float *X,
                                      const int incX, const float beta, float *Y, const int incY, void *stream);

/* ------------------------------------------------------- banded level 2 */
/* test/level2/sgbmv/exo_sgbmv.h:5-23, dgbmv likewise: y = beta y + alpha A x,
 * A an M x N band (KL sub-, KU super-diagonals) in row-major band storage
 * (row i holds columns i-KL .. i+KU); no Order / Trans argument */
EXOBLAS_API void exo_sgbmv(const int M, const int N, const int KL, const int KU, const float alpha, const float *A,
               const int lda, const float *X, const int incX, const float beta, float *Y, const int incY);
EXOBLAS_API void exo_dgbmv(const int M, const int N, const int KL, const int KU, const double alpha, const double *A,
               const int lda, const double *X, const int incX, const double beta, double *Y, const int incY);
/* test/level2/ssbmv/exo_ssbmv.h:7-52: y = beta y + alpha A x, A symmetric with K off-diagonals */
EXOBLAS_API void exo_ssbmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const int K,
               const float alpha, const float *A, const int lda, const float *X, const int incX, const float beta,
               float *Y, const int incY);
EXOBLAS_API void exo_dsbmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const int N, const int K,
               const double alpha, const double *A, const int lda, const double *X, const int incX, const double beta,
               double *Y, const int incY);
/* test/level2/stbmv/exo_stbmv.h: x = op(A) x, A triangular with K off-diagonals */
EXOBLAS_API void exo_stbmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const int K, const float *A, const int lda, float *X,
               const int incX);
EXOBLAS_API void exo_dtbmv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const int K, const double *A, const int lda, double *X,
               const int incX);
/* test/level2/stbsv/exo_stbsv.h: solve op(A) x = b in place, A triangular banded */
EXOBLAS_API void exo_stbsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const int K, const float *A, const int lda, float *X,
               const int incX);
EXOBLAS_API void exo_dtbsv(const enum CBLAS_ORDER order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE TransA,
               const enum CBLAS_DIAG Diag, const int N, const int K, const double *A, const int lda, double *X,
               const int incX);

/* ------------------------------------------------------------ level 3 --- */
/* test/level3/gemm/exo_gemm_wrapper.h:9-28 (C *= beta, then C += alpha op(A) op(B)) */
EXOBLAS_API void exo_sgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TransA, const enum CBLAS_TRANSPOSE TransB,
               const int M, const int N, const int K, const float alpha, const float *A, const int lda, const float *B,
               const int ldb, const float beta, float *C, const int ldc);
EXOBLAS_API void exo_dgemm(const enum CBLAS_ORDER Order, const enum CBLAS_TRANSPOSE TransA, const enum CBLAS_TRANSPOSE TransB,
               const int M, const int N, const int K, const double alpha, const double *A, const int lda,
               const double *B, const int ldb, const double beta, double *C, const int ldc);
/* test/level3/symm/exo_symm_wrapper.h:9-27 */
EXOBLAS_API void exo_ssymm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo, const int M,
               const int N, const float alpha, const float *A, const int lda, const float *B, const int ldb,
               const float beta, float *C, const int ldc);
EXOBLAS_API void exo_dsymm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo, const int M,
               const int N, const double alpha, const double *A, const int lda, const double *B, const int ldb,
               const double beta, double *C, const int ldc);
/* test/level3/syrk/exo_syrk_wrapper.h:9-28 (the triangle of C *= beta, then the update) */
EXOBLAS_API void exo_ssyrk(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans, const int N,
               const int K, const float alpha, const float *A, const int lda, const float beta, float *C,
               const int ldc);
EXOBLAS_API void exo_dsyrk(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans, const int N,
               const int K, const double alpha, const double *A, const int lda, const double beta, double *C,
               const int ldc);
/* test/level3/syr2k/exo_syr2k_wrapper.h:9-32 (the triangle of C *= beta, then
 * C_tri += alpha (op(A) op(B)^T + op(B) op(A)^T)) */
EXOBLAS_API void exo_ssyr2k(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans,
               const int N, const int K, const float alpha, const float *A, const int lda, const float *B,
               const int ldb, const float beta, float *C, const int ldc);
EXOBLAS_API void exo_dsyr2k(const enum CBLAS_ORDER Order, const enum CBLAS_UPLO Uplo, const enum CBLAS_TRANSPOSE Trans,
               const int N, const int K, const double alpha, const double *A, const int lda, const double *B,
               const int ldb, const double beta, double *C, const int ldc);
/* test/level3/strmm/exo_strmm.h:7-58 (B = alpha op(A) B, A triangular, Side
 * Left; like the reference, Side Right leaves B unchanged) */
EXOBLAS_API void exo_strmm(const enum CBLAS_ORDER Order, const enum CBLAS_SIDE Side, const enum CBLAS_UPLO Uplo,
               const enum CBLAS_TRANSPOSE TransA, const enum CBLAS_DIAG Diag, const int M, const int N,
               const float alpha, const float *A, const int lda, float *B, const int ldb);

/* ------------------------------------------------------------ batching --- */
/* Many independent exo_sgemm / exo_dgemv / exo_strsv calls of uneven sizes
 * in one persistent launch (no counterpart in the reference, whose calls run
 * one at a time on the calling thread).  All operands are device pointers.
 *   SGEMM: flags = {TransA, TransB}, m, n, k, alpha, beta, A/lda, B/ldb, C/ldc (float)
 *   DGEMV: flags = {TransA}, m = M, n = N, alpha, beta, A/lda, B = X (ldb = incX),
 *          C = Y (ldc = incY) (double)
 *   STRSV: flags = {Uplo, TransA, Diag}, m = N (<= 4096), A/lda, C = X (ldc = incX) (float)
 * Semantics per call are those of the corresponding exo_* entry point.  A
 * plan uploads the calls once; runs queue one persistent kernel on the
 * thread's stream (blocking mode waits for it), after the grouped
 * tensor-core product of the large sgemm calls (below); graph launches
 * replay a captured CUDA graph of that run.  sgemm tile shapes come from the
 * autotuner (exoblas_batch_tune; cached in the JSON file named by
 * EXOBLAS_TUNE_CACHE when set). */
enum EXOBLAS_BATCH_OPCODE { EXOBLAS_BATCH_SGEMM = 1, EXOBLAS_BATCH_DGEMV = 2, EXOBLAS_BATCH_STRSV = 3 };
typedef struct exoblas_batch_op {
  int op;
  int flags[3];
  int m, n, k;
  double alpha, beta;
  const void *A;
  int lda;
  const void *B;
  int ldb;
  void *C;
  int ldc;
} exoblas_batch_op;
typedef struct exoblas_batch_plan_s *exoblas_batch_plan;
EXOBLAS_API int exoblas_batch_plan_create(const exoblas_batch_op *ops, int count, exoblas_batch_plan *plan);
EXOBLAS_API int exoblas_batch_plan_run(exoblas_batch_plan plan);
EXOBLAS_API int exoblas_batch_plan_graph_launch(exoblas_batch_plan plan);
EXOBLAS_API int exoblas_batch_plan_info(exoblas_batch_plan plan, int *units, double *flops, double *bytes);
EXOBLAS_API int exoblas_batch_plan_destroy(exoblas_batch_plan plan);
EXOBLAS_API int exoblas_batch_tune(void);
/* tile configuration the autotuner picked for an sgemm of this shape (0: 32x32, 1: 64x64, 2: 128x128) */
EXOBLAS_API int exoblas_batch_tile_config(int m, int n, int k);
/* sgemm calls with m, n and k all >= 128 run on the tensor cores, as one
 * grouped split-BF16 product per plan (FP32 operands as three BF16 terms
 * each, the exo_sgemm split-BF16 path: error at or below FFMA's); on by
 * default.  Off: every call on the FFMA work units.  Applies to plans created
 * afterwards (process-wide). */
EXOBLAS_API int exoblas_batch_set_tensor_cores(int on);
/* number of the plan's calls on the tensor cores */
EXOBLAS_API int exoblas_batch_plan_tensor_core_calls(exoblas_batch_plan plan, int *calls);

/* ------------------------------------------------------------- serving --- */
/* A request server with continuous batching (no counterpart in the
 * reference).  Small requests (gemm / syrk with m n k <= 2^24, gemv with
 * m n <= 2^22, trsv with n <= 512) are gathered by a batcher thread: each
 * tick runs every small request that arrived since the previous tick as one
 * device batch (one launch over all their tiles, row blocks and solves;
 * FFMA / DFMA tiles for gemm and syrk), and requests arriving meanwhile join
 * the next tick.  Larger requests go to W worker threads, each with its own
 * stream and workspace; such a request is admitted when a worker is free and
 * its estimated device-memory footprint fits in the admission budget with
 * everything in flight.  Device batches and worker requests overlap on the
 * device.  Operands are device pointers.  On the worker path,
 * single-precision gemm / syrk run the split-BF16 path, double gemm / syrk
 * the Ozaki path, gemv / trsv their kernels.
 *   GEMM: flags = {TransA, TransB}, m, n, k, A/lda, B/ldb, C/ldc
 *   SYRK: flags = {Uplo, Trans}, m = N, k = K, A/lda, C/ldc
 *   GEMV: flags = {TransA}, m = M, n = N, A/lda, B = X (ldb = incX), C = Y (ldc = incY)
 *   TRSV: flags = {Uplo, TransA, Diag}, m = N, A/lda, C = X (ldc = incX)
 * precision: 1 single, 2 double.  Arrivals beyond the queue capacity are
 * rejected and counted. */
enum EXOBLAS_REQUEST_OP { EXOBLAS_REQ_GEMM = 1, EXOBLAS_REQ_GEMV = 2, EXOBLAS_REQ_TRSV = 3, EXOBLAS_REQ_SYRK = 4 };
typedef struct exoblas_request {
  int op;
  int precision;
  int flags[3];
  int m, n, k;
  double alpha, beta;
  const void *A;
  int lda;
  const void *B;
  int ldb;
  void *C;
  int ldc;
} exoblas_request;
typedef struct exoblas_server_s *exoblas_server;
/* hbm_budget_bytes = 0: 70% of the free device memory; queue_capacity = 0:
 * unbounded; scratch_reserve_bytes: workspace each worker allocates up front */
EXOBLAS_API int exoblas_server_create(int workers, size_t hbm_budget_bytes, size_t queue_capacity,
                                      size_t scratch_reserve_bytes, exoblas_server *server);
/* arrival_s on the exoblas_server_now() clock (< 0: now) */
EXOBLAS_API int exoblas_server_submit(exoblas_server server, const exoblas_request *request, double arrival_s);
EXOBLAS_API double exoblas_server_now(void);
/* submits requests[i] at t0 + offsets_s[i], t0 = the call's start (written
 * to *t0_out when not NULL); returns once the last one is submitted */
EXOBLAS_API int exoblas_server_replay(exoblas_server server, const exoblas_request *requests, const double *offsets_s,
                                      size_t count, double *t0_out);
EXOBLAS_API int exoblas_server_drain(exoblas_server server);
/* stats[0..7]: completed, rejected, failed, p50 latency s, p99 s, mean s,
 * max s, completed per second (first arrival to last completion) */
EXOBLAS_API int exoblas_server_stats(exoblas_server server, double *stats);
/* Continuous batching of small requests: stats[0..2] = requests served by
 * device batches, device batches run, mean requests per batch. */
EXOBLAS_API int exoblas_server_batch_stats(exoblas_server server, double *stats);
EXOBLAS_API int exoblas_server_destroy(exoblas_server server);
/* grows the calling thread's device workspace to at least `bytes` now */
EXOBLAS_API int exoblas_reserve_scratch(size_t bytes);

#ifdef __cplusplus
}
#endif

#endif /* EXOBLAS_GB300_H */
