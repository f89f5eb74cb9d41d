"""Batched persistent execution (exoblas_batch_* in include/exoblas.h).

    plan = BatchPlan([BatchOp.sgemm(...), BatchOp.dgemv(...), BatchOp.strsv(...)])
    plan.run()            # one persistent launch on the library's stream
    plan.graph_launch()   # the same run replayed from a captured CUDA graph

Operands are device addresses (ints) or CUDA torch tensors.
"""
from __future__ import annotations

import ctypes as C

from . import _native
from .blas import ExoBlasError, _ptr

SGEMM, DGEMV, STRSV = 1, 2, 3


class BatchOp(C.Structure):
    _fields_ = [
        ("op", C.c_int),
        ("flags", C.c_int * 3),
        ("m", C.c_int),
        ("n", C.c_int),
        ("k", C.c_int),
        ("alpha", C.c_double),
        ("beta", C.c_double),
        ("A", C.c_void_p),
        ("lda", C.c_int),
        ("B", C.c_void_p),
        ("ldb", C.c_int),
        ("C", C.c_void_p),
        ("ldc", C.c_int),
    ]

    @classmethod
    def sgemm(cls, transa, transb, m, n, k, alpha, A, lda, B, ldb, beta, Cm, ldc):
        return cls(SGEMM, (C.c_int * 3)(transa, transb, 0), m, n, k, alpha, beta, _ptr(A), lda, _ptr(B), ldb,
                   _ptr(Cm), ldc)

    @classmethod
    def dgemv(cls, trans, m, n, alpha, A, lda, x, incx, beta, y, incy):
        return cls(DGEMV, (C.c_int * 3)(trans, 0, 0), m, n, 0, alpha, beta, _ptr(A), lda, _ptr(x), incx, _ptr(y),
                   incy)

    @classmethod
    def strsv(cls, uplo, trans, diag, n, A, lda, x, incx):
        return cls(STRSV, (C.c_int * 3)(uplo, trans, diag), n, 0, 0, 1.0, 0.0, _ptr(A), lda, None, 0, _ptr(x), incx)


def tune() -> None:
    st = _native.lib().exoblas_batch_tune()
    if st:
        raise ExoBlasError(st, "exoblas_batch_tune")


def tile_config(m, n, k) -> int:
    return _native.lib().exoblas_batch_tile_config(m, n, k)


def set_tensor_cores(on: bool) -> None:
    """sgemm calls with m, n, k >= 128 on the tensor cores (split-BF16) in
    plans created afterwards; off: every call on FFMA work units."""
    st = _native.lib().exoblas_batch_set_tensor_cores(1 if on else 0)
    if st:
        raise ExoBlasError(st, "exoblas_batch_set_tensor_cores")


class BatchPlan:
    def __init__(self, ops):
        arr = (BatchOp * len(ops))(*ops)
        self._arr = arr
        h = C.c_void_p()
        st = _native.lib().exoblas_batch_plan_create(C.cast(arr, C.c_void_p), len(ops), C.byref(h))
        if st:
            raise ExoBlasError(st, "exoblas_batch_plan_create")
        self.handle = h

    def info(self):
        u, f, b = C.c_int(), C.c_double(), C.c_double()
        _native.lib().exoblas_batch_plan_info(self.handle, C.byref(u), C.byref(f), C.byref(b))
        return {"units": u.value, "flops": f.value, "bytes": b.value}

    def tensor_core_calls(self) -> int:
        n = C.c_int()
        st = _native.lib().exoblas_batch_plan_tensor_core_calls(self.handle, C.byref(n))
        if st:
            raise ExoBlasError(st, "exoblas_batch_plan_tensor_core_calls")
        return n.value

    def run(self):
        st = _native.lib().exoblas_batch_plan_run(self.handle)
        if st:
            raise ExoBlasError(st, "exoblas_batch_plan_run")

    def graph_launch(self):
        st = _native.lib().exoblas_batch_plan_graph_launch(self.handle)
        if st:
            raise ExoBlasError(st, "exoblas_batch_plan_graph_launch")

    def close(self):
        if self.handle:
            _native.lib().exoblas_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
