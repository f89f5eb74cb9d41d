"""CPU checks of the oracle itself (no GPU).

1. Pin: the oracle reproduces the committed CBLAS (OpenBLAS) outputs of the
   golden fixtures under the reference's own 1% rule, within the
   componentwise FP64 bound, and bit-exactly for copy/swap/scal(+-1).
2. The reference's deterministic trsv fixture (A = 2.0, X[i] = i).
3. The wrapper special cases the oracle restates.
4. A planted mistake in the oracle is caught by the same checks.
"""
import numpy as np
import pytest

import golden_io
from common import EPS, assert_bound, assert_rel1pct, fp64_reference, run_oracle

FIXTURES = [(name, i) for name in golden_io.names() for i in range(len(golden_io.load(name)))]
_cache = {}


def fixture(name, i):
    if name not in _cache:
        _cache[name] = golden_io.load(name)
    return _cache[name][i]


def check_against(case, got_r, got_args, exp_r, exp_out, what):
    if case.exact:
        if case.scalar:
            assert got_r == exp_r, f"{what}: {case} result {got_r} != {exp_r}"
        for j, e in exp_out.items():
            assert got_args[j].tobytes() == e.tobytes(), f"{what}: {case} output {j} not bit-exact"
        return
    if case.op.endswith("trsv") or case.op.endswith("tbsv"):
        for j, e in exp_out.items():
            assert_rel1pct(got_args[j], e, f"{what} {case}")
        return
    (r64, a64), (m, am) = fp64_reference(case)
    if case.scalar:
        assert_rel1pct([got_r], [exp_r], f"{what} {case}")
        if case.op in ("dsdot", "sdsdot"):
            # OpenBLAS 0.3.31's dsdot accumulates in FP32 on this host, so it is
            # held to the FP32 bound; the oracle must meet the FP64 one
            # (dsdot.py:11-21 accumulates in f64).
            assert_bound([exp_r], [r64], [m], case.nred, "s", 8.0, f"cblas {case} vs fp64")
            assert_bound([got_r], [r64], [m], case.nred, case.p, 8.0, f"{what} {case} vs fp64")
        else:
            assert_bound([got_r], [exp_r], [m], case.nred, case.p, 8.0, f"{what} {case} vs cblas")
    for j, e in exp_out.items():
        assert_rel1pct(got_args[j], e, f"{what} {case} out{j}")
        assert_bound(got_args[j], e, am[j], case.nred, case.p, 8.0, f"{what} {case} out{j} vs cblas")


@pytest.mark.parametrize("name,i", FIXTURES, ids=lambda v: str(v))
def test_oracle_matches_cblas_golden(name, i):
    case, exp_r, exp_out = fixture(name, i)
    r, a = run_oracle(case)
    check_against(case, r, a, exp_r, exp_out, "oracle")


def test_trsv_reference_fixture():
    """test/level2/trsv/correctness.cpp:20-25: every A entry is 2.0 (2 + j/N in
    integer arithmetic), X[i] = i; the exact lower solution is x = [0, .5, .5, ...]."""
    import oracle

    for n in (2, 100, 321):
        A = np.full(n * n, 2.0)
        x = np.arange(n, dtype=np.float64)
        oracle.call("dtrsv", 101, 122, 111, 131, n, A, n, x, 1)
        exp = np.r_[0.0, np.full(n - 1, 0.5)]
        np.testing.assert_allclose(x, exp, rtol=0, atol=1e-12)


def test_wrapper_special_cases():
    import oracle

    x = np.arange(1, 6, dtype=np.float32)
    assert oracle.call("sasum", 5, x, -1) == 0.0  # exo_asum_wrapper.h:14-16
    y = x.copy()
    oracle.call("sscal", 5, 3.0, y, -1)  # exo_scal_wrapper.h:23-25
    assert np.array_equal(y, x)
    oracle.call("sscal", 5, 0.0, y, 1)  # scal_alpha_0 writes zeros
    assert not y.any()
    y = x.copy()
    oracle.call("saxpy", 5, 0.0, x, 1, y, 1)  # exo_axpy_wrapper.h:8-10
    assert np.array_equal(y, x)
    P = np.array([-2.0, 1, 2, 3, 4], np.float32)  # rotm flag -2: no branch taken
    a, b = x.copy(), x[::-1].copy()
    oracle.call("srotm", 5, a, 1, b, 1, P)
    assert np.array_equal(a, x) and np.array_equal(b, x[::-1])
    C = np.ones(4, np.float32)
    oracle.call("sgemm", 102, 111, 111, 2, 2, 2, 1.0, C, 2, C, 2, 0.0, C.copy(), 2)
    assert oracle.last_status() == 1  # Order != RowMajor: the reference throws


def test_planted_mistake_is_caught():
    """An oracle output perturbed by 2% in one element fails the 1% rule and
    the componentwise bound (the checks are not vacuous)."""
    case, exp_r, exp_out = fixture("gemv", 0)
    r, a = run_oracle(case)
    j = case.outputs[0]
    a[j] = a[j].copy()
    a[j][0] = a[j][0] * 1.02 + 0.02
    with pytest.raises(AssertionError):
        check_against(case, r, a, exp_r, exp_out, "planted")


def test_double_double_dot_is_exact_on_cancellation():
    """Dot2 recovers a sum that cancels catastrophically in plain FP64."""
    import oracle

    x = np.array([1e16, 1.0, -1e16, 1.0])
    y = np.ones(4)
    assert oracle.call("dd_dot", 4, x, 1, y, 1) == 2.0
