"""CPU checks of the oracle itself (no GPU).

1. Pin: the oracle reproduces the committed CBLAS (OpenBLAS) outputs of the
   golden fixtures under the reference's own 1% rule, within the
   componentwise FP64 bound, and bit-exactly for copy/swap/scal(+-1).
2. The reference's deterministic trsv fixture (A = 2.0, X[i] = i).
3. The wrapper special cases the oracle restates.
4. A planted mistake in the oracle is caught by the same checks.
5. The double-word instantiation (the d-precision reference): exact to the
   last bit on small cases checked in rational arithmetic, within the bound
   of every d-precision golden fixture, and the FP64 oracle within the bound
   of it.
"""
import numpy as np
import pytest

import golden_io
from common import assert_bound, assert_rel1pct, fp64_reference, run_dw, run_oracle, to64

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


D_FIXTURES = [(n, i) for n, i in FIXTURES if fixture(n, i)[0].p == "d" and not fixture(n, i)[0].exact]


@pytest.mark.parametrize("name,i", D_FIXTURES, ids=lambda v: str(v))
def test_double_word_reference_pins(name, i):
    """Every d-precision fixture: the double-word restatement meets CBLAS's
    outputs (1% rule, componentwise bound), and the plain FP64 oracle meets
    the double-word result within the bound."""
    case, exp_r, exp_out = fixture(name, i)
    hp = run_dw(to64(case))
    if hp is None:
        pytest.skip(f"{case.op}: no double-word variant (exact or index result)")
    (r, a), (m, am) = hp, fp64_reference(case)[1]
    o_r, o_a = run_oracle(case)
    tri_solve = case.op.endswith("trsv") or case.op.endswith("tbsv")
    if case.scalar:
        assert_rel1pct([r], [exp_r], f"dw {case}")
        # OpenBLAS's dsdot accumulates in FP32 on this host: the FP32 bound
        pcb = "s" if case.op == "dsdot" else "d"
        assert_bound([exp_r], [r], [m], case.nred, pcb, 8.0, f"cblas {case} vs dw")
        assert_bound([o_r], [r], [m], case.nred, "d", 8.0, f"oracle {case} vs dw")
    for j, e in exp_out.items():
        assert_rel1pct(a[j], e, f"dw {case} out{j}")
        if not tri_solve:  # a solve's forward error is not held to a product bound
            assert_bound(e, a[j], am[j], case.nred, "d", 8.0, f"cblas {case} out{j} vs dw")
            assert_bound(o_a[j], a[j], am[j], case.nred, "d", 8.0, f"oracle {case} out{j} vs dw")


def test_double_word_is_correctly_rounded_on_small_cases():
    """dgemv, ddot and dtrsv (a unit lower matrix with integer entries, whose
    solution is exact in rationals) in double-word arithmetic against exact
    rational arithmetic: the rounded result is within half an ulp."""
    from fractions import Fraction as F

    import oracle

    g = np.random.default_rng(5)
    A = g.uniform(-1, 1, (23, 31))
    x = g.uniform(-1, 1, 31)
    y = g.uniform(-1, 1, 23)
    _, out = oracle.call_dw("dgemv", 101, 111, 23, 31, 0.7, A, 31, x, 1, -0.3, y, 1)
    for i in range(23):
        ex = F(-0.3) * F(y[i]) + sum(F(0.7) * (F(x[j]) * F(A[i, j])) for j in range(31))
        assert abs(F(out[10][i]) - ex) <= F(np.spacing(abs(float(ex)))) / 2
    r, _ = oracle.call_dw("ddot", 31, x, 1, x[::-1].copy(), 1)
    ex = sum(F(a) * F(b) for a, b in zip(x, x[::-1]))
    assert abs(F(r) - ex) <= F(np.spacing(abs(float(ex)))) / 2
    n = 12
    L = np.tril(g.integers(-3, 4, (n, n)).astype(np.float64), -1) + np.eye(n)
    b = g.uniform(-1, 1, n)
    _, out = oracle.call_dw("dtrsv", 101, 122, 111, 132, n, L, n, b, 1)
    xs = []
    for i in range(n):
        xs.append(F(b[i]) - sum(F(L[i, j]) * xs[j] for j in range(i)))
    for i in range(n):
        assert abs(F(out[7][i]) - xs[i]) <= F(np.spacing(abs(float(xs[i])))) / 2


def test_double_word_keeps_nan_and_infinity():
    """beta = 0 keeps a NaN of C (mscal multiplies) and an infinite input stays
    infinite rather than turning into the NaN of a low-part cancellation."""
    import oracle

    C = np.array([np.nan, 1.0, 2.0, 3.0])
    A = np.ones(4)
    _, out = oracle.call_dw("dgemm", 101, 111, 111, 2, 2, 2, 1.0, A, 2, A, 2, 0.0, C, 2)
    assert np.isnan(out[12][0]) and np.array_equal(out[12][1:], [2.0, 2.0, 2.0])
    y = np.array([1.0, np.inf])
    _, out = oracle.call_dw("daxpy", 2, 2.0, np.ones(2), 1, y, 1)
    assert out[4][0] == 3.0 and out[4][1] == np.inf
