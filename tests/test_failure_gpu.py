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
