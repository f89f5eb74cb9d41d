"""Request server with continuous batching (exoblas_server_* in include/exoblas.h)."""
from __future__ import annotations

import ctypes as C

from . import _native
from .blas import ExoBlasError, _ptr

GEMM, GEMV, TRSV, SYRK = 1, 2, 3, 4
SINGLE, DOUBLE = 1, 2


class Request(C.Structure):
    _fields_ = [
        ("op", C.c_int),
        ("precision", C.c_int),
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


def request(op, precision, flags=(0, 0, 0), m=0, n=0, k=0, alpha=1.0, beta=0.0, A=None, lda=0, B=None, ldb=0,
            Cm=None, ldc=0):
    f = (C.c_int * 3)(*(list(flags) + [0, 0, 0])[:3])
    return Request(op, precision, f, m, n, k, alpha, beta, _ptr(A), lda, _ptr(B), ldb, _ptr(Cm), ldc)


def _chk(st, name):
    if st:
        raise ExoBlasError(st, name)


class Server:
    def __init__(self, workers=8, hbm_budget=0, queue_capacity=0, scratch_reserve=0):
        h = C.c_void_p()
        _chk(_native.lib().exoblas_server_create(workers, hbm_budget, queue_capacity, scratch_reserve, C.byref(h)),
             "exoblas_server_create")
        self.handle = h

    @staticmethod
    def now():
        return _native.lib().exoblas_server_now()

    def submit(self, req, arrival=-1.0):
        _chk(_native.lib().exoblas_server_submit(self.handle, C.byref(req), arrival), "exoblas_server_submit")

    def replay(self, reqs, offsets):
        """Submits reqs[i] at t0 + offsets[i] seconds; returns t0."""
        n = len(reqs)
        arr = (Request * n)(*reqs)
        off = (C.c_double * n)(*[float(v) for v in offsets])
        t0 = C.c_double()
        _chk(_native.lib().exoblas_server_replay(self.handle, C.cast(arr, C.c_void_p), C.cast(off, C.c_void_p), n,
                                                 C.byref(t0)), "exoblas_server_replay")
        return t0.value

    def drain(self):
        _chk(_native.lib().exoblas_server_drain(self.handle), "exoblas_server_drain")

    def batch_stats(self):
        """Requests served by device batches, batches run, mean requests per batch."""
        s = (C.c_double * 3)()
        _chk(_native.lib().exoblas_server_batch_stats(self.handle, s), "exoblas_server_batch_stats")
        return {"batched": int(s[0]), "batches": int(s[1]), "per_batch": s[2]}

    def stats(self):
        s = (C.c_double * 8)()
        _chk(_native.lib().exoblas_server_stats(self.handle, s), "exoblas_server_stats")
        keys = ["completed", "rejected", "failed", "p50_s", "p99_s", "mean_s", "max_s", "solves_per_s"]
        return dict(zip(keys, list(s)))

    def close(self):
        if self.handle:
            _native.lib().exoblas_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
