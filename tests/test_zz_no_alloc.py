"""exoblas_sgemv_noalloc: the sgemv entry point for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

Called through the C ABI twice in a row, each result is checked against an
FP64 matvec of the same inputs within the componentwise bound the other GPU
tests use (c = 4), and against the regular exo_sgemv on the same inputs
within the bound between two such results (c = 8).  Also covered: an empty x
with a NaN alpha (y = beta y, as exo_sgemv), a Trans call whose packed x
leaves room for fewer column-sum chunks than exo_sgemv uses, column-major
calls with the per-thread opt-in, and the rejection of problems beyond the
array.  This file sorts last so that a run stopping at the first failure has
already run every other test; it also passes alone.
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


def _strided(v, inc, n):
    """The n logical entries of a strided vector, in logical order."""
    out = v[::abs(inc)][:n].astype(np.float64)
    return out[::-1] if inc < 0 else out


def _check_fp64(A, lda, trans, M, N, alpha, X, incX, beta, Y0, incY, got, c=4.0):
    """|got - (alpha op(A) x + beta y)| <= c (xlen + 1) eps_s magnitude, in FP64."""
    xlen, ylen = (M, N) if trans == 112 else (N, M)
    A2 = A.reshape(M, lda)[:, :N].astype(np.float64)
    op = A2.T if trans == 112 else A2
    x, y0 = _strided(X, incX, xlen), _strided(Y0, incY, ylen)
    ref = alpha * (op @ x) + beta * y0
    mag = abs(alpha) * (np.abs(op) @ np.abs(x)) + abs(beta) * np.abs(y0)
    g = _strided(got, incY, ylen)
    err = np.abs(g - ref)
    tol = c * (xlen + 1) * EPS["s"] * mag
    assert np.all(err <= tol), f"max err/tol {float(np.max(err / np.maximum(tol, 1e-300)))}"
    return mag


@pytest.mark.gpu
def test_noalloc_sgemv_matches_fp64_and_exo_sgemv_twice(cuda):
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
        got = y_new.cpu().numpy()
        mag = _check_fp64(A, lda, trans, M, N, 1.5, X, incX, 0.5, Y, incY, got)
        # against exo_sgemv: the bound between two results within c = 4 each
        a = _strided(y_ref.cpu().numpy(), incY, ylen)
        b = _strided(got, incY, ylen)
        assert np.all(np.abs(a - b) <= 8 * (xlen + 1) * EPS["s"] * mag)
        # elements between the strided entries of y are left as they were
        mask = np.ones(Y.size, bool)
        mask[::abs(incY)] = False
        assert np.array_equal(got[mask], Y[mask])


@pytest.mark.gpu
def test_noalloc_empty_x_scales_y_by_beta_only(cuda):
    """N = 0 with NoTrans (x is empty): y = beta y without touching alpha, so
    a NaN alpha leaves y finite, exactly as exo_sgemv."""
    import exoblas_gb300 as eb
    from exoblas_gb300 import _native

    torch = cuda
    L = _native.lib()
    Y = np.linspace(-1, 1, 50, dtype=np.float32)
    A = torch.zeros(4, device="cuda")
    for beta in (0.5, 0.0):
        y_ref = torch.from_numpy(Y).cuda()
        y_new = torch.from_numpy(Y).cuda()
        eb.exo_sgemv(101, 111, 50, 0, float("nan"), A, 1, A, 1, beta, y_ref, 1)
        st = _noalloc(L, torch, 101, 111, 50, 0, float("nan"), A, 1, A, 1, beta, y_new, 1)
        assert st == 0
        assert torch.equal(y_new, y_ref)
        assert torch.equal(y_new, torch.from_numpy(beta * Y).cuda())


@pytest.mark.gpu
def test_noalloc_fewer_chunks_than_exo_sgemv_stays_in_bound(cuda):
    """Trans with M = 1,040,000 rows and a strided x: the packed x takes
    4,160,000 of the 4 MiB, leaving room for 67 chunks of N = 128 column sums
    where exo_sgemv would use more.  The result is held to the FP64 bound."""
    from exoblas_gb300 import _native

    torch = cuda
    L = _native.lib()
    M, N, incX = 1_040_000, 128, 2
    gen = torch.Generator(device="cuda").manual_seed(3)
    dA = torch.rand(M * N, device="cuda", generator=gen).mul_(2).sub_(1)
    dX = torch.rand(1 + (M - 1) * incX, device="cuda", generator=gen).mul_(2).sub_(1)
    y0 = torch.rand(N, device="cuda", generator=gen).mul_(2).sub_(1)
    y = y0.clone()
    st = _noalloc(L, torch, 101, 112, M, N, 1.25, dA, N, dX, incX, -0.5, y, 1)
    assert st == 0, L.exoblas_status_string(st)
    Ad, x = dA.view(M, N).double(), dX[::incX].double()
    ref = 1.25 * (Ad.t() @ x) - 0.5 * y0.double()
    mag = 1.25 * (Ad.abs().t() @ x.abs()) + 0.5 * y0.double().abs()
    err = (y.double() - ref).abs()
    assert bool((err <= 4 * (M + 1) * EPS["s"] * mag).all())
    del dA, dX


@pytest.mark.gpu
def test_noalloc_column_major_follows_exo_sgemv(cuda):
    """Rejected like exo_sgemv by default; with the per-thread column-major
    opt-in, the same column-major call as exo_sgemv within the bound."""
    import exoblas_gb300 as eb
    from exoblas_gb300 import _native

    torch = cuda
    L = _native.lib()
    g = np.random.default_rng(12)
    M, N, lda = 300, 200, 305  # column-major: lda >= M
    A = g.uniform(-1, 1, N * lda).astype(np.float32)
    dA = torch.from_numpy(A).cuda()
    for trans in (111, 112):
        xlen, ylen = (N, M) if trans == 111 else (M, N)
        dX = torch.from_numpy(g.uniform(-1, 1, xlen).astype(np.float32)).cuda()
        y0 = torch.from_numpy(g.uniform(-1, 1, ylen).astype(np.float32)).cuda()
        y = y0.clone()
        assert _noalloc(L, torch, 102, trans, M, N, 1.0, dA, lda, dX, 1, 0.25, y, 1) != 0
        assert torch.equal(y, y0)
        L.exoblas_set_column_major(1)
        try:
            y_ref = y0.clone()
            eb.exo_sgemv(102, trans, M, N, 1.0, dA, lda, dX, 1, 0.25, y_ref, 1)
            st = _noalloc(L, torch, 102, trans, M, N, 1.0, dA, lda, dX, 1, 0.25, y, 1)
        finally:
            L.exoblas_set_column_major(0)
        assert st == 0, L.exoblas_status_string(st)
        Acm = dA.view(N, lda)[:, :M].t().double()  # the M x N column-major matrix
        op = Acm if trans == 111 else Acm.t()
        mag = op.abs() @ dX.double().abs() + 0.25 * y0.double().abs()
        ref = op @ dX.double() + 0.25 * y0.double()
        assert bool(((y.double() - ref).abs() <= 4 * (xlen + 1) * EPS["s"] * mag).all())
        assert bool(((y.double() - y_ref.double()).abs() <= 8 * (xlen + 1) * EPS["s"] * mag).all())


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
