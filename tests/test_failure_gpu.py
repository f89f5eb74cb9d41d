"""Failure detection on the GPU without a fault: a bounded wait that runs out.

The trsv solvers, the batch kernel and the tcgen05 kernels bound every wait
and, on expiry, record it in the device status word and return; the host
then reports EXOBLAS_TIMEOUT.  exoblas_selftest_wait_timeout launches one
kernel whose flag nothing sets, so its wait expires after the given time
through that same path.  The context must stay usable afterwards.
"""
import ctypes as C

import numpy as np
import pytest

from exoblas_gb300 import _native

EXOBLAS_SUCCESS = 0
EXOBLAS_INVALID_VALUE = 2
EXOBLAS_TIMEOUT = 5


@pytest.mark.gpu
def test_expired_wait_reports_timeout_and_context_survives():
    L = _native.lib()
    assert L.exoblas_selftest_wait_timeout(0.02) == EXOBLAS_TIMEOUT
    assert L.exoblas_get_status() == EXOBLAS_TIMEOUT
    # the status word was cleared: the next synchronisation is clean
    assert L.exoblas_synchronize() == EXOBLAS_SUCCESS
    # and ordinary calls on the same thread's context still run and are right
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, 4097).astype(np.float32)
    y = rng.uniform(-1, 1, 4097).astype(np.float32)
    r = L.exo_sdot(x.size, x.ctypes.data_as(C.c_void_p), 1, y.ctypes.data_as(C.c_void_p), 1)
    assert L.exoblas_get_status() == EXOBLAS_SUCCESS
    ref = float(np.dot(x.astype(np.float64), y.astype(np.float64)))
    assert abs(r - ref) <= 4 * x.size * np.finfo(np.float32).eps * float(np.abs(x) @ np.abs(y))
    # a second expiry behaves the same
    assert L.exoblas_selftest_wait_timeout(0.01) == EXOBLAS_TIMEOUT
    assert L.exoblas_synchronize() == EXOBLAS_SUCCESS


@pytest.mark.gpu
def test_selftest_rejects_out_of_range_waits():
    L = _native.lib()
    for s in (0.0, -1.0, 2.0, float("nan")):
        assert L.exoblas_selftest_wait_timeout(s) == EXOBLAS_INVALID_VALUE


EXOBLAS_UNSUPPORTED_ORDER = 1


@pytest.mark.gpu
def test_error_statuses_handler_and_untouched_outputs():
    """The reference throws on a non-RowMajor Order; the C ABI instead records
    a per-thread status, calls the installed handler and leaves every output
    untouched.  Arguments that would make a kernel go out of bounds (negative
    sizes, lda below the row length) are rejected the same way."""
    L = _native.lib()
    seen = []
    HANDLER = C.CFUNCTYPE(None, C.c_int, C.c_char_p, C.c_char_p)
    handler = HANDLER(lambda st, fn, msg: seen.append((st, fn.decode(), msg.decode())))
    L.exoblas_set_error_handler(C.cast(handler, C.c_void_p))
    try:
        m = 8
        A = np.ones((m, m), np.float32)
        B = np.ones((m, m), np.float32)
        Cm = np.full((m, m), 7.0, np.float32)
        ptr = lambda a: a.ctypes.data_as(C.c_void_p)
        # Order != RowMajor (column-major calls are opt-in and off here)
        L.exo_sgemm(102, 111, 111, m, m, m, 1.0, ptr(A), m, ptr(B), m, 0.0, ptr(Cm), m)
        assert L.exoblas_get_status() == EXOBLAS_UNSUPPORTED_ORDER
        assert (Cm == 7.0).all()
        assert seen and seen[-1][0] == EXOBLAS_UNSUPPORTED_ORDER and seen[-1][1] == "exo_sgemm"
        # lda smaller than the row length
        L.exo_sgemm(101, 111, 111, m, m, m, 1.0, ptr(A), m - 1, ptr(B), m, 0.0, ptr(Cm), m)
        assert L.exoblas_get_status() == EXOBLAS_INVALID_VALUE and (Cm == 7.0).all()
        # negative size
        x = np.ones(16, np.float32)
        y = np.full(16, 3.0, np.float32)
        L.exo_saxpy(-1, 2.0, ptr(x), 1, ptr(y), 1)
        assert L.exoblas_get_status() == EXOBLAS_INVALID_VALUE and (y == 3.0).all()
        assert len(seen) == 3 and all(msg for _, _, msg in seen)
        # a successful call resets the status and does not call the handler
        L.exo_saxpy(16, 2.0, ptr(x), 1, ptr(y), 1)
        assert L.exoblas_get_status() == EXOBLAS_SUCCESS and (y == 5.0).all() and len(seen) == 3
    finally:
        L.exoblas_set_error_handler(None)
    for st in range(7):
        s = L.exoblas_status_string(st)
        assert isinstance(s, bytes) and len(s) > 0
