"""Level-3 parity on the GPU (grids of test/level3/{gemm,symm,syrk,syr2k,strmm}/correctness.cpp)."""
import numpy as np
import pytest

from cases import gemm_cases, symm_cases, syr2k_cases, syrk_cases, trmm_cases
from common import EPS, check_case, run_gpu

GEMM = [c for p in "sd" for c in gemm_cases(p)]
SYMM = [c for p in "sd" for c in symm_cases(p)]
SYRK = [c for p in "sd" for c in syrk_cases(p)]
SYR2K = [c for p in "sd" for c in syr2k_cases(p)][::2]
TRMM = list(trmm_cases())


@pytest.mark.gpu
@pytest.mark.parametrize("case", GEMM, ids=lambda c: f"{c.op}-{c.label}")
def test_gemm(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", SYMM, ids=lambda c: f"{c.op}-{c.label}")
def test_symm(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", SYRK, ids=lambda c: f"{c.op}-{c.label}")
def test_syrk(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", SYR2K, ids=lambda c: f"{c.op}-{c.label}")
def test_syr2k(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", TRMM, ids=lambda c: f"{c.op}-{c.label}")
def test_strmm(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
def test_strmm_right_side_and_order(cuda):
    """Side Right leaves B unchanged and a column-major call is rejected, as
    in test/level3/strmm/exo_strmm.h:12-14, 45-56."""
    import exoblas_gb300 as eb

    g = np.random.default_rng(3)
    A = g.uniform(-1, 1, 16 * 16).astype(np.float32)
    B = g.uniform(-1, 1, 16 * 8).astype(np.float32)
    B0 = B.copy()
    eb.exo_strmm(101, 142, 121, 111, 131, 16, 8, 1.5, A, 16, B, 8)
    assert B.tobytes() == B0.tobytes()
    with pytest.raises(eb.UnsupportedParameterException):
        eb.exo_strmm(102, 141, 121, 111, 131, 16, 8, 1.5, A, 16, B, 8)


@pytest.mark.gpu
def test_sgemm_config_1024(cuda):
    """Config: sgemm NN 1024^3, lda=ldb=ldc=1024, alpha 1, beta 0.5, U[-1,1) seed 0."""
    import exoblas_gb300 as eb

    g = np.random.default_rng(0)
    n = 1024
    A = g.uniform(-1, 1, (n, n)).astype(np.float32)
    B = g.uniform(-1, 1, (n, n)).astype(np.float32)
    C = g.uniform(-1, 1, (n, n)).astype(np.float32)
    out = C.copy()
    eb.exo_sgemm(101, 111, 111, n, n, n, 1.0, A, n, B, n, 0.5, out, n)
    ref = A.astype(np.float64) @ B.astype(np.float64) + 0.5 * C.astype(np.float64)
    mag = np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64)) + 0.5 * np.abs(C.astype(np.float64))
    assert np.all(np.abs(out - ref) <= 4 * n * EPS["s"] * mag)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_beta_zero_multiplies_c(cuda, mode):
    """Level 3 scales C by beta as a multiplication even when beta == 0
    (src/level3/mscal.py:12-28), so a NaN in C stays NaN; every precision
    path (native, split-BF16, Ozaki) keeps that."""
    import exoblas_gb300 as eb

    g = np.random.default_rng(23)
    m, n, k = 70, 66, 40
    eb.set_precision(mode)
    try:
        for p, dt in (("s", np.float32), ("d", np.float64)):
            A = g.uniform(-1, 1, (m, k)).astype(dt)
            B = g.uniform(-1, 1, (k, n)).astype(dt)
            C = g.uniform(-1, 1, (m, n)).astype(dt)
            C[5, 9] = np.nan
            getattr(eb, f"exo_{p}gemm")(101, 111, 111, m, n, k, 1.0, A, k, B, n, 0.0, C, n)
            assert np.isnan(C[5, 9]) and np.isfinite(np.delete(C.ravel(), 5 * n + 9)).all()

            S = g.uniform(-1, 1, (m, m)).astype(dt)
            C = g.uniform(-1, 1, (m, n)).astype(dt)
            C[7, 3] = np.nan
            Bs = g.uniform(-1, 1, (m, n)).astype(dt)
            getattr(eb, f"exo_{p}symm")(101, 141, 121, m, n, 1.0, S, m, Bs, n, 0.0, C, n)
            assert np.isnan(C[7, 3]) and np.isfinite(np.delete(C.ravel(), 7 * n + 3)).all()

            Ak = g.uniform(-1, 1, (m, k)).astype(dt)
            C = g.uniform(-1, 1, (m, m)).astype(dt)
            C[9, 2] = np.nan   # inside the lower triangle
            C[1, 8] = np.nan   # outside it: left alone
            getattr(eb, f"exo_{p}syrk")(101, 122, 111, m, k, 1.0, Ak, k, 0.0, C, m)
            assert np.isnan(C[9, 2]) and np.isnan(C[1, 8])
            mask = np.ones_like(C, dtype=bool)
            mask[9, 2] = mask[1, 8] = False
            assert np.isfinite(C[mask & np.tril(np.ones_like(mask))]).all()
    finally:
        eb.set_precision(0)


def _fp32_bound(got, ref, mag, k):
    """|got - ref| <= 4 (k + 1) eps_s |A||B| componentwise (FP64 reference)."""
    err = (got.double() - ref).abs()
    return bool((err <= 4 * (k + 1) * EPS["s"] * mag + 1e-300).all())


@pytest.mark.gpu
@pytest.mark.parametrize("ta", [111, 112])
@pytest.mark.parametrize("tb", [111, 112])
def test_sgemm_full_tile_path(cuda, ta, tb):
    """sgemm on the FP32 full-tile path (m, n multiples of 128 with at least
    one tile per SM, k a multiple of 16), every transpose pair, against FP64."""
    import exoblas_gb300 as eb

    torch = cuda
    eb.set_precision(eb.PRECISION_NATIVE)
    m, n, k = 2048, 1536, 272
    g = torch.Generator(device="cuda").manual_seed(ta * 7 + tb)
    A = torch.rand(m * k, device="cuda", generator=g).mul_(2).sub_(1)
    B = torch.rand(k * n, device="cuda", generator=g).mul_(2).sub_(1)
    C0 = torch.rand(m * n, device="cuda", generator=g).mul_(2).sub_(1)
    C = C0.clone()
    lda, ldb = (k if ta == 111 else m), (n if tb == 111 else k)
    eb.exo_sgemm(101, ta, tb, m, n, k, 1.25, A, lda, B, ldb, -0.5, C, n)
    opA = A.view(m, k) if ta == 111 else A.view(k, m).t()
    opB = B.view(k, n) if tb == 111 else B.view(n, k).t()
    ref = 1.25 * (opA.double() @ opB.double()) - 0.5 * C0.view(m, n).double()
    mag = 1.25 * (opA.double().abs() @ opB.double().abs()) + 0.5 * C0.view(m, n).double().abs()
    assert _fp32_bound(C.view(m, n), ref, mag, k)


@pytest.mark.gpu
@pytest.mark.parametrize("uplo", [121, 122])
@pytest.mark.parametrize("trans", [111, 112])
def test_ssyrk_full_tile_path(cuda, uplo, trans):
    """ssyrk on the full-tile path: the triangle against FP64, the other
    triangle untouched."""
    import exoblas_gb300 as eb

    torch = cuda
    eb.set_precision(eb.PRECISION_NATIVE)
    n, k = 2048, 144
    g = torch.Generator(device="cuda").manual_seed(uplo + trans)
    A = torch.rand(n * k, device="cuda", generator=g).mul_(2).sub_(1)
    C0 = torch.rand(n * n, device="cuda", generator=g).mul_(2).sub_(1)
    C = C0.clone()
    eb.exo_ssyrk(101, uplo, trans, n, k, 0.75, A, k if trans == 111 else n, 0.5, C, n)
    opA = (A.view(n, k) if trans == 111 else A.view(k, n).t()).double()
    ref = 0.75 * (opA @ opA.t()) + 0.5 * C0.view(n, n).double()
    mag = 0.75 * (opA.abs() @ opA.abs().t()) + 0.5 * C0.view(n, n).double().abs()
    tri = torch.triu(torch.ones(n, n, dtype=torch.bool, device="cuda"))
    if uplo == 122:
        tri = tri.t()
    Cv = C.view(n, n)
    assert _fp32_bound(Cv[tri], ref[tri], mag[tri], k)
    assert torch.equal(Cv[~tri], C0.view(n, n)[~tri])


@pytest.mark.gpu
@pytest.mark.parametrize("side", [141, 142])
@pytest.mark.parametrize("uplo", [121, 122])
def test_ssymm_full_tile_path(cuda, side, uplo):
    """ssymm on the full-tile path (sym(A) written out from the stored
    triangle, then the FP32 tiles); the unstored triangle of A holds NaN and
    must not be read."""
    import exoblas_gb300 as eb

    torch = cuda
    eb.set_precision(eb.PRECISION_NATIVE)
    m, n = 2048, 1280
    d = m if side == 141 else n
    g = torch.Generator(device="cuda").manual_seed(side + uplo)
    A = torch.rand(d, d, device="cuda", generator=g).mul_(2).sub_(1)
    stored = torch.triu(A) if uplo == 121 else torch.tril(A)
    S = (stored + stored.t() - torch.diag(torch.diag(A))).double()
    Anan = A.clone()
    hidden = torch.tril(torch.ones(d, d, dtype=torch.bool, device="cuda"), -1)
    Anan[hidden if uplo == 121 else hidden.t()] = float("nan")
    B = torch.rand(m, n, device="cuda", generator=g).mul_(2).sub_(1)
    C0 = torch.rand(m, n, device="cuda", generator=g).mul_(2).sub_(1)
    C = C0.clone()
    eb.exo_ssymm(101, side, uplo, m, n, 1.5, Anan.flatten(), d, B.flatten(), n, 0.25, C.view(-1), n)
    Bd = B.double()
    prod, pmag = (S @ Bd, S.abs() @ Bd.abs()) if side == 141 else (Bd @ S, Bd.abs() @ S.abs())
    ref = 1.5 * prod + 0.25 * C0.double()
    mag = 1.5 * pmag + 0.25 * C0.double().abs()
    assert _fp32_bound(C, ref, mag, d)
