"""Shared parity machinery for the tests.

Every BLAS entry point here has the same C signature in three places: the GPU
library (exo_<p><op>), the CPU oracle (oracle_<p><op>) and CBLAS
(scipy_cblas_<p><op>).  A Case holds one argument list in that order with
NumPy buffers filled the way the reference's AlignedBuffer fills them
(1 + (N-1)|inc| elements, uniform[-1, 1), test/common/generate_buffer.h:
12-78), but from a seeded PCG64 generator so runs reproduce.

Checks, in the order the reference and the project's accuracy contract
define them:
- the reference's own rule, |r - e| / max(1, |e|) < 1% on every element of
  every output buffer, padding included (test/common/correctness_helpers.h:
  9-16, generate_buffer.h:57-68);
- the componentwise bound |r - e| <= c * n * eps * m, where e is an FP64
  result for s-precision and a double-word (about 104-bit) result for
  d-precision, n the reduction length and m the same operation evaluated on
  absolute values (|alpha||A||x| + |beta||y| for gemv, and so on);
- bit-exactness for copy, swap and scal by +-1.
"""
from __future__ import annotations

import copy as _copy
from dataclasses import dataclass, field

import numpy as np

ROW, COL = 101, 102
NT, TR = 111, 112
UP, LO = 121, 122
NU, UN = 131, 132
LEFT, RIGHT = 141, 142

DT = {"s": np.float32, "d": np.float64}
EPS = {"s": float(np.finfo(np.float32).eps), "d": float(np.finfo(np.float64).eps)}


def rng(seed):
    return np.random.default_rng(seed)


def buf(g, n, inc, dtype):
    """AlignedBuffer(N, inc): 1 + (N-1)|inc| uniform[-1,1) values."""
    size = 1 + (max(n, 1) - 1) * abs(inc)
    return g.uniform(-1.0, 1.0, size).astype(dtype)


def mat(g, rows, ld, dtype):
    """AlignedBuffer2D(rows, ld) flattened."""
    return g.uniform(-1.0, 1.0, max(rows, 1) * ld).astype(dtype)


@dataclass
class Case:
    op: str  # e.g. "sgemv"
    args: list
    outputs: list  # indices of output buffers in args
    scalar: bool = False  # the call returns the result
    nred: int = 1  # reduction length for the bound
    exact: bool = False  # bit-exact expected (copy, swap, scal +-1)
    label: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def p(self):
        return self.op[0] if self.op not in ("dsdot", "sdsdot") else ("d" if self.op == "dsdot" else "s")

    def clone_args(self):
        return [a.copy() if isinstance(a, np.ndarray) else a for a in self.args]

    def __repr__(self):
        return f"Case({self.op} {self.label})"


def run_oracle(case: Case):
    import oracle

    a = case.clone_args()
    r = oracle.call(case.op, *a)
    return r, a


def run_cblas(case: Case):
    from oracle import cblas

    a = case.clone_args()
    if case.op.endswith("gbmv"):  # exo_?gbmv has no Order / TransA: row-major NoTrans
        r = cblas.call(case.op, ROW, 111, *a)
    else:
        r = cblas.call(case.op, *a)
    return r, a


def run_gpu(case: Case, device: bool = False):
    """Run exo_<op>.  device=True moves every buffer to a CUDA torch tensor."""
    import exoblas_gb300 as eb

    a = case.clone_args()
    if device:
        import torch

        dev = [torch.from_numpy(v).cuda() if isinstance(v, np.ndarray) else v for v in a]
        r = getattr(eb, "exo_" + case.op)(*dev)
        torch.cuda.synchronize()
        a = [d.cpu().numpy() if isinstance(v, np.ndarray) else v for v, d in zip(a, dev)]
    else:
        r = getattr(eb, "exo_" + case.op)(*a)
    return r, a


def to64(case: Case) -> Case:
    """The same case with every buffer and scalar promoted to float64 (the
    'd' variant of the op), used as the FP64 oracle for s-precision."""
    c = _copy.copy(case)
    c.args = [a.astype(np.float64) if isinstance(a, np.ndarray) else a for a in case.args]
    if case.op in ("dsdot", "sdsdot"):
        c.op = "ddot" if case.op == "dsdot" else "ddot"
        if case.op == "sdsdot":
            c.args = c.args[:1] + c.args[2:]
            c.extra = dict(case.extra, sb=case.args[1])
    elif case.op[0] == "s":
        c.op = "d" + case.op[1:]
    return c


def magnitude_case(case64: Case) -> Case:
    """Same op on absolute values: per element this yields the componentwise
    magnitude |alpha||A||x| + |beta||y| (gemv), |c||x| + |s||y| (rot), ..."""
    c = _copy.copy(case64)
    args = []
    for a in case64.args:
        if isinstance(a, np.ndarray):
            args.append(np.abs(a))
        elif isinstance(a, float):
            args.append(abs(a))
        else:
            args.append(a)
    c.args = args
    return c


def rel1pct_ok(r, e) -> np.ndarray:
    """test/common/correctness_helpers.h:9-16"""
    r = np.asarray(r, np.float64)
    e = np.asarray(e, np.float64)
    return np.abs(r - e) / np.maximum(1.0, np.abs(e)) < 0.01


def assert_rel1pct(r, e, what=""):
    ok = rel1pct_ok(r, e)
    if not np.all(ok):
        i = int(np.argmin(ok))
        raise AssertionError(f"{what}: 1% rule fails at {i}: got {np.ravel(r)[i]!r} expected {np.ravel(e)[i]!r}")


def assert_bound(r, e, mag, n, p, c=4.0, what=""):
    """|r - e| <= c * n * eps * mag (+ a tiny absolute floor for zeros)."""
    r = np.asarray(r, np.float64).ravel()
    e = np.asarray(e, np.float64).ravel()
    mag = np.asarray(mag, np.float64).ravel()
    eps = EPS[p]
    tol = c * max(n, 1) * eps * mag + 8 * np.finfo(np.float64).tiny
    err = np.abs(r - e)
    bad = ~(err <= tol) & ~(np.isnan(r) & np.isnan(e))
    if np.any(bad):
        i = int(np.flatnonzero(bad)[0])
        raise AssertionError(
            f"{what}: componentwise bound fails at {i}: got {r[i]!r} expected {e[i]!r} "
            f"err {err[i]:.3e} > tol {tol[i]:.3e} (c={c}, n={n}, eps={eps:.2e})"
        )


def _magnitude(c64: Case):
    """Oracle run on absolute values.  rot and rotm carry signs inside their
    formulas (y' = -s x + c y, y' = -x + h22 y), so their magnitudes are
    assembled from sign-adjusted runs instead."""
    if c64.op == "drot":
        a = magnitude_case(c64)
        _, ax = run_oracle(a)
        b = _copy.copy(a)
        b.args = list(a.args)
        b.args[6] = -abs(c64.args[6])
        _, ay = run_oracle(b)
        ax[3] = ay[3]
        return None, ax
    if c64.op == "drotm":
        P = c64.args[5]
        flag, h11, h21, h12, h22 = P
        eff = {-1.0: (h11, h21, h12, h22), 0.0: (1.0, h21, h12, 1.0), 1.0: (h11, 1.0, 1.0, h22)}.get(float(flag))
        a = magnitude_case(c64)
        if eff is not None:
            a.args[5] = np.array([-1.0, *map(abs, eff)], np.float64)
        else:
            a.args[5] = P.copy()
        return run_oracle(a)
    return run_oracle(magnitude_case(c64))


def run_dw(case64: Case):
    """The oracle's double-word instantiation of a d-op (about 104 significand
    bits), rounded to double; None when the op has none (exact ops, iamax)."""
    import oracle

    if case64.op not in oracle.DW_OPS:
        return None
    return oracle.call_dw(case64.op, *case64.clone_args())


def fp64_reference(case: Case):
    """High-precision result and FP64 magnitude for a case.

    s-precision (and sdsdot): the oracle's d-variant in FP64, whose own
    rounding is far below the FP32 bound.  d-precision (and dsdot): the same
    restated loop nest in double-word arithmetic, so the FP64 result under
    test is measured against a reference that does not carry FP64 rounding.
    The magnitude (the op on absolute values) is an FP64 run either way; it
    only scales the bound."""
    c64 = to64(case)
    hp = run_dw(c64) if case.p == "d" else None
    r64, a64 = hp if hp is not None else run_oracle(c64)
    m, am = _magnitude(c64)
    if case.op == "sdsdot":
        r64 = r64 + case.args[1]
        m = m + abs(case.args[1])
    return (r64, a64), (m, am)


def check_case(case: Case, got_r, got_args, c=4.0, what="gpu"):
    """Check a result (scalar or output buffers) against the oracle with the
    1% rule and against FP64 with the componentwise bound (or bit-exactly)."""
    o_r, o_args = run_oracle(case)
    if case.exact:
        for i in case.outputs:
            assert got_args[i].tobytes() == o_args[i].tobytes(), f"{what}: {case} output {i} not bit-exact"
        return
    (r64, a64), (m, am) = fp64_reference(case)
    p = case.p
    if case.scalar:
        assert_rel1pct([got_r], [o_r], f"{what} {case}")
        assert_bound([got_r], [r64], [m], case.nred, p, c, f"{what} {case}")
    for i in case.outputs:
        assert_rel1pct(got_args[i], o_args[i], f"{what} {case} out{i}")
        assert_bound(got_args[i], a64[i], am[i], case.nred, p, c, f"{what} {case} out{i}")


def _tr_product(op, args, xs, d_prec):
    """op(A) xs for a triangular (dtrmv) or banded triangular (dtbmv) matrix:
    double-word for d-precision, so the residual carries no FP64 rounding of
    its own; FP64 for s-precision."""
    import oracle

    if d_prec:
        _, out = oracle.call_dw(op, *args[:-2], xs, args[-1])
        return out[-2]
    r = xs.copy()
    oracle.call(op, *args[:-2], r, args[-1])
    return r


def trsv_residual_ok(case: Case, xhat: np.ndarray, c=8.0):
    """|b - op(A) xhat| <= c n eps |op(A)| |xhat| componentwise.  The product
    op(A) xhat is formed in double-word for dtrsv and FP64 for strsv."""
    import oracle

    order, u, t, d, n, A, lda, x, inc = case.args
    step = abs(inc)
    b = x.astype(np.float64)[::step][:n]
    xs = xhat.astype(np.float64)[::step][:n]
    if inc < 0:
        b, xs = b[::-1].copy(), xs[::-1].copy()
    A64 = A.astype(np.float64)
    r = _tr_product("dtrmv", [order, u, t, d, n, A64, lda, None, 1], xs, case.p == "d")
    m = np.abs(xs)
    oracle.call("dtrmv", order, u, t, d, n, np.abs(A64), lda, m, 1)
    eps = EPS[case.p]
    bad = np.abs(b - r) > c * max(n, 1) * eps * m + 1e-300
    assert not bad.any(), f"{case}: residual bound fails at {np.flatnonzero(bad)[:5]}"


def tbsv_residual_ok(case: Case, xhat: np.ndarray, c=8.0):
    """|b - op(A) xhat| <= c (k + 1) eps |op(A)| |xhat| componentwise, the
    product in double-word for dtbsv and FP64 for stbsv."""
    import oracle

    order, u, t, d, n, k, A, lda, x, inc = case.args
    A64 = A.astype(np.float64)
    xs = xhat.astype(np.float64).copy()
    r = _tr_product("dtbmv", [order, u, t, d, n, k, A64, lda, None, inc], xs, case.p == "d")
    m = np.abs(xhat.astype(np.float64))
    oracle.call("dtbmv", order, u, t, d, n, k, np.abs(A64), lda, m, inc)
    b = x.astype(np.float64)
    sel = np.arange(0, 1 + (n - 1) * abs(inc), abs(inc))
    bad = np.abs(b[sel] - r[sel]) > c * (k + 1) * EPS[case.p] * m[sel] + 1e-300
    assert not bad.any(), f"{case}: residual bound fails at {np.flatnonzero(bad)[:5]}"
