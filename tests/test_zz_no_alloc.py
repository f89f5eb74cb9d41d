"""exoblas_sgemv_noalloc: the sgemv entry point for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

Called through the C ABI twice in a row, each result is checked against the
regular exo_sgemv on the same inputs within the componentwise bound the
other GPU tests use.  This file sorts last so that a run stopping at the
first failure has already run every other test; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest

from common import EPS


def _noalloc(L, torch, order, trans, M, N, alpha, A, lda, X, incX, beta, Y, incY):
    s = torch.cuda.current_stream().cuda_stream
    st = L.exoblas_sgemv_noalloc(order, trans, M, N, alpha, C.c_void_p(A.data_ptr()), lda, C.c_void_p(X.data_ptr()),
                                 incX, beta, C.c_void_p(Y.data_ptr()), incY, C.c_void_p(s) if s else None)
    torch.cuda.synchronize()
    return st


@pytest.mark.gpu
def test_noalloc_sgemv_matches_exo_sgemv_twice(cuda):
    import exoblas_gb300 as eb
    from exoblas_gb300 import _native

    torch = cuda
    L = _native.lib()
    g = np.random.default_rng(11)
    # two calls in a row: Trans with a strided x (uses the partial sums and
    # the packed x), then NoTrans with a negative y stride
    calls = [(112, 1000, 3000, 2, 1), (111, 777, 2049, 1, -3)]
    for trans, M, N, incX, incY in calls:
        lda = N + 3
        xlen, ylen = (M, N) if trans == 112 else (N, M)
        A = g.uniform(-1, 1, M * lda).astype(np.float32)
        X = g.uniform(-1, 1, 1 + (xlen - 1) * abs(incX)).astype(np.float32)
        Y = g.uniform(-1, 1, 1 + (ylen - 1) * abs(incY)).astype(np.float32)
        dA, dX = torch.from_numpy(A).cuda(), torch.from_numpy(X).cuda()
        y_ref, y_new = torch.from_numpy(Y).cuda(), torch.from_numpy(Y).cuda()
        eb.exo_sgemv(101, trans, M, N, 1.5, dA, lda, dX, incX, 0.5, y_ref, incY)
        st = _noalloc(L, torch, 101, trans, M, N, 1.5, dA, lda, dX, incX, 0.5, y_new, incY)
        assert st == 0, L.exoblas_status_string(st)
        # componentwise bound (c = 4 per result, so 8 between two results)
        A2 = A.reshape(M, lda)[:, :N].astype(np.float64)
        op = A2.T if trans == 112 else A2
        xs = np.abs(X[::abs(incX)][:xlen].astype(np.float64))
        if incX < 0:
            xs = xs[::-1]
        ys = np.abs(Y[::abs(incY)][:ylen].astype(np.float64))
        if incY < 0:
            ys = ys[::-1]
        mag = 1.5 * (np.abs(op) @ xs) + 0.5 * ys
        a = y_ref.cpu().numpy()[::abs(incY)][:ylen].astype(np.float64)
        b = y_new.cpu().numpy()[::abs(incY)][:ylen].astype(np.float64)
        if incY < 0:
            a, b, = a[::-1], b[::-1]
        assert np.all(np.abs(a - b) <= 8 * xlen * EPS["s"] * mag)
        # elements between the strided entries of y are left as they were
        mask = np.ones(Y.size, bool)
        mask[::abs(incY)] = False
        assert np.array_equal(y_new.cpu().numpy()[mask], Y[mask])


@pytest.mark.gpu
def test_noalloc_rejects_problems_beyond_its_scratch(cuda):
    from exoblas_gb300 import _native

    torch = cuda
    L = _native.lib()
    A = torch.zeros(16, device="cuda")
    X = torch.zeros(16, device="cuda")
    Y = torch.ones(16, device="cuda")
    # Trans with N = 2^21 columns needs 8 MiB of partial sums > 4 MiB
    st = _noalloc(L, torch, 101, 112, 4, 1 << 21, 1.0, A, 1 << 21, X, 1, 0.0, Y, 1)
    assert st == 2  # EXOBLAS_INVALID_VALUE, nothing queued
    assert torch.all(Y == 1)
