"""Ozaki slice emulation of dgemm / dsymm / dsyrk on tcgen05 tensor cores.

Results must meet the FP64 componentwise bound against the double-double
oracle (the reference grid of test/level3/gemm/correctness.cpp in double,
and a larger case with sampled entries), stay bit-for-bit deterministic, and
fall back to the FP64 FMA kernel when an input is not finite (NaN / inf
propagate as in the reference)."""
import numpy as np
import pytest

from cases import gemm_cases, symm_cases, syr2k_cases, syrk_cases
from common import EPS, check_case, run_gpu


@pytest.fixture
def ozaki_mode(cuda):
    import exoblas_gb300 as eb

    eb.set_precision(eb.PRECISION_OZAKI)
    yield
    eb.set_precision(eb.PRECISION_NATIVE)


CASES = ([c for c in gemm_cases("d", dims=(1, 7, 64, 257), ldds=(0, 5))][::3]
         + [c for c in symm_cases("d", dims=(1, 7, 64, 257))][::2]
         + [c for c in syrk_cases("d", dims=(1, 7, 64, 257, 300))][::2]
         + [c for c in syr2k_cases("d", dims=(1, 7, 64, 257), ldds=(0, 5))][::8])


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c.op}-{c.label}")
def test_ozaki_grid(ozaki_mode, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("stress", [False, True])
def test_ozaki_against_double_double(ozaki_mode, stress):
    import exoblas_gb300 as eb
    import oracle

    g = np.random.default_rng(5 if stress else 4)
    m, n, k = 1000, 900, 1500
    if stress:
        A = g.choice([-1.0, 1.0], (m, k)) * g.uniform(1, 2, (m, k)) * np.exp2(g.integers(-16, 17, (m, k)))
        B = g.choice([-1.0, 1.0], (k, n)) * g.uniform(1, 2, (k, n)) * np.exp2(g.integers(-16, 17, (k, n)))
    else:
        A = g.uniform(-1, 1, (m, k))
        B = g.uniform(-1, 1, (k, n))
    C0 = g.uniform(-1, 1, (m, n))
    C = C0.copy()
    eb.exo_dgemm(101, 111, 111, m, n, k, 1.5, A, k, B, n, 0.25, C, n)
    rows = g.integers(0, m, 400).astype(np.int64)
    cols = g.integers(0, n, 400).astype(np.int64)
    ref = np.zeros(400)
    oracle.call("dd_gemm_entries", 0, 0, k, 1.5, A, k, B, n, 0.25, C0, n, rows, cols, 400, ref)
    mag = 1.5 * np.einsum("ik,ki->i", np.abs(A[rows]), np.abs(B[:, cols])) + 0.25 * np.abs(C0[rows, cols])
    err = np.abs(C[rows, cols] - ref)
    assert np.all(err <= 4 * k * EPS["d"] * mag), float((err / mag).max())


@pytest.mark.gpu
def test_ozaki_deterministic_and_nonfinite_fallback(ozaki_mode):
    import exoblas_gb300 as eb

    g = np.random.default_rng(6)
    A = g.uniform(-1, 1, (300, 200))
    B = g.uniform(-1, 1, (200, 250))
    outs = []
    for _ in range(2):
        C = np.zeros((300, 250))
        eb.exo_dgemm(101, 111, 111, 300, 250, 200, 1.0, A, 200, B, 250, 0.0, C, 250)
        outs.append(C)
    assert outs[0].tobytes() == outs[1].tobytes()
    A[3, 7] = np.nan
    C = np.zeros((300, 250))
    eb.exo_dgemm(101, 111, 111, 300, 250, 200, 1.0, A, 200, B, 250, 0.0, C, 250)
    assert np.isnan(C[3]).all() and np.isfinite(np.delete(C, 3, axis=0)).all()
