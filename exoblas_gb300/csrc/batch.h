// Batched execution internals shared by batch.cu and the request server.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace exb {
namespace bt {

// One call of a device batch: the batch API's exoblas_batch_op normalised,
// or a request the server batches.  op: EXOBLAS_BATCH_SGEMM / _DGEMV /
// _STRSV or one of the server's op codes below.
struct Op {
  int op;
  int f0, f1, f2;  // gemm: transA, transB; gemv: trans; trsv: uplo, trans, diag
  int tri;         // gemm tiles: 0 all of C, 1 its lower triangle, 2 its upper (syrk)
  int m, n, k;     // trsv: order m
  double alpha, beta;
  const void *A;
  long lda;
  const void *B;  // gemv: x
  long ldb;       // gemv: incx
  void *C;        // gemv: y; trsv: x
  long ldc;       // gemv: incy; trsv: incx
};

// Server op codes (beside EXOBLAS_BATCH_SGEMM = 1, _DGEMV = 2, _STRSV = 3).
// A syrk is a gemm of op(A) with op(A)^T restricted to one triangle (tri).
enum ServerOp : int { kOpDGemm = 11, kOpSSyrk = 12, kOpDSyrk = 13, kOpSGemv = 14, kOpDTrsv = 15 };

struct TickRunner;
TickRunner *tick_create();
void tick_destroy(TickRunner *t);
// Runs one device batch of `ops` (all operands device pointers) on the
// runner's stream and waits for it; false on an unknown op code.
bool tick_run(TickRunner *t, const std::vector<Op> &ops, int sm_count);

}  // namespace bt
}  // namespace exb
