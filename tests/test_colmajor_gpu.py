"""Column-major calls (exoblas_set_column_major, off by default as in the
reference, which rejects them): each op's column-major result against an
FP64 NumPy evaluation of the column-major definition, within the same
componentwise bound the row-major paths meet.  The NumPy side reads the
buffers as column-major arrays directly, so it shares nothing with the
library's row-major mapping."""
import numpy as np
import pytest

from common import EPS

COL = 102
NT, TR = 111, 112
UP, LO = 121, 122
NU, UN = 131, 132
LEFT, RIGHT = 141, 142


def cm(buf, rows, cols, ld):
    """rows x cols view of column-major storage with leading dimension ld."""
    return buf[: ld * cols].reshape(cols, ld)[:, :rows].T


def vec(buf, n, inc):
    v = buf[:: abs(inc)][:n]
    return v[::-1] if inc < 0 else v


def tri(A, upper, unit):
    T = np.triu(A) if upper else np.tril(A)
    if unit:
        np.fill_diagonal(T, 1.0)
    return T


def sym(A, upper):
    T = np.triu(A) if upper else np.tril(A)
    return T + T.T - np.diag(np.diag(A))


def check(got, ref, mag, n, p, what):
    got = np.asarray(got, np.float64)
    tol = 4 * max(n, 1) * EPS[p] * np.abs(mag) + 1e-300
    bad = np.abs(got - ref) > tol
    assert not bad.any(), f"{what}: max err {np.max(np.abs(got - ref))} at {np.argwhere(bad)[:3]}"


@pytest.fixture
def colmajor(cuda):
    import exoblas_gb300 as eb

    eb.set_column_major(True)
    yield eb
    eb.set_column_major(False)


DT = {"s": np.float32, "d": np.float64}


@pytest.mark.gpu
@pytest.mark.parametrize("p", "sd")
@pytest.mark.parametrize("ta,tb", [(NT, NT), (NT, TR), (TR, NT), (TR, TR)])
def test_gemm_colmajor(colmajor, p, ta, tb):
    eb, g = colmajor, np.random.default_rng(1)
    m, n, k, ldd = 37, 29, 41, 3
    ar, ac = (m, k) if ta == NT else (k, m)
    br, bc = (k, n) if tb == NT else (n, k)
    lda, ldb, ldc = ar + ldd, br + ldd, m + ldd
    A, B = g.uniform(-1, 1, lda * ac).astype(DT[p]), g.uniform(-1, 1, ldb * bc).astype(DT[p])
    C = g.uniform(-1, 1, ldc * n).astype(DT[p])
    A64, B64, C64 = (cm(A.astype(np.float64), ar, ac, lda), cm(B.astype(np.float64), br, bc, ldb),
                     cm(C.astype(np.float64), m, n, ldc))
    opA, opB = (A64 if ta == NT else A64.T), (B64 if tb == NT else B64.T)
    ref = 1.5 * opA @ opB + 0.5 * C64
    mag = 1.5 * np.abs(opA) @ np.abs(opB) + 0.5 * np.abs(C64)
    getattr(eb, f"exo_{p}gemm")(COL, ta, tb, m, n, k, 1.5, A, lda, B, ldb, 0.5, C, ldc)
    check(cm(C, m, n, ldc), ref, mag, k + 1, p, "gemm")


@pytest.mark.gpu
@pytest.mark.parametrize("p", "sd")
@pytest.mark.parametrize("t", [NT, TR])
def test_gemv_ger_colmajor(colmajor, p, t):
    eb, g = colmajor, np.random.default_rng(2)
    m, n, lda = 53, 31, 60
    A = g.uniform(-1, 1, lda * n).astype(DT[p])
    xl, yl = (n, m) if t == NT else (m, n)
    x, y = g.uniform(-1, 1, 2 * xl).astype(DT[p]), g.uniform(-1, 1, yl).astype(DT[p])
    A64 = cm(A.astype(np.float64), m, n, lda)
    opA = A64 if t == NT else A64.T
    xv = vec(x.astype(np.float64), xl, -2)
    ref = 0.75 * opA @ xv + 0.5 * y.astype(np.float64)
    mag = 0.75 * np.abs(opA) @ np.abs(xv) + 0.5 * np.abs(y.astype(np.float64))
    getattr(eb, f"exo_{p}gemv")(COL, t, m, n, 0.75, A, lda, x, -2, 0.5, y, 1)
    check(y, ref, mag, xl + 1, p, "gemv")
    # ger: A += alpha x y^T (M x N column-major)
    x2, y2 = g.uniform(-1, 1, m).astype(DT[p]), g.uniform(-1, 1, n).astype(DT[p])
    A0 = cm(A.astype(np.float64), m, n, lda).copy()
    ref = A0 + 1.25 * np.outer(x2, y2)
    getattr(eb, f"exo_{p}ger")(COL, m, n, 1.25, x2, 1, y2, 1, A, lda)
    check(cm(A, m, n, lda), ref, np.abs(A0) + 1.25 * np.abs(np.outer(x2, y2)), 2, p, "ger")


@pytest.mark.gpu
@pytest.mark.parametrize("p", "sd")
@pytest.mark.parametrize("u", [UP, LO])
def test_symmetric_level2_colmajor(colmajor, p, u):
    eb, g = colmajor, np.random.default_rng(3)
    n, lda = 45, 50
    A = g.uniform(-1, 1, lda * n).astype(DT[p])
    x, y = g.uniform(-1, 1, n).astype(DT[p]), g.uniform(-1, 1, n).astype(DT[p])
    S = sym(cm(A.astype(np.float64), n, n, lda), u == UP)
    ref = 1.5 * S @ x + 0.5 * y
    mag = 1.5 * np.abs(S) @ np.abs(x.astype(np.float64)) + 0.5 * np.abs(y.astype(np.float64))
    getattr(eb, f"exo_{p}symv")(COL, u, n, 1.5, A, lda, x, 1, 0.5, y, 1)
    check(y, ref, mag, n + 1, p, "symv")
    # syr2: triangle of A += alpha (x y^T + y x^T); the other triangle untouched
    A0 = cm(A.astype(np.float64), n, n, lda).copy()
    upd = 0.5 * (np.outer(x, y) + np.outer(y, x))
    keep = np.triu(np.ones((n, n), bool)) if u == UP else np.tril(np.ones((n, n), bool))
    ref = np.where(keep, A0 + upd, A0)
    getattr(eb, f"exo_{p}syr2")(COL, u, n, 0.5, x, 1, y, 1, A, lda)
    check(cm(A, n, n, lda), ref, np.abs(A0) + np.abs(upd), 3, p, "syr2")


@pytest.mark.gpu
@pytest.mark.parametrize("p", "sd")
@pytest.mark.parametrize("u,t,d", [(UP, NT, NU), (LO, TR, UN), (UP, TR, NU), (LO, NT, UN)])
def test_triangular_colmajor(colmajor, p, u, t, d):
    eb, g = colmajor, np.random.default_rng(4)
    n, lda = 70, 75
    A = (g.uniform(-1, 1, lda * n) / n).astype(DT[p])
    A64 = cm(A.astype(np.float64), n, n, lda)
    for i in range(n):
        A[i * lda + i] = 1 + g.uniform(0, 1)
    A64 = cm(A.astype(np.float64), n, n, lda)
    T = tri(A64, u == UP, d == UN)
    opT = T if t == NT else T.T
    x = g.uniform(-1, 1, n).astype(DT[p])
    ref = opT @ x.astype(np.float64)
    xm = x.copy()
    getattr(eb, f"exo_{p}trmv")(COL, u, t, d, n, A, lda, xm, 1)
    check(xm, ref, np.abs(opT) @ np.abs(x.astype(np.float64)), n + 1, p, "trmv")
    b = x.copy()
    getattr(eb, f"exo_{p}trsv")(COL, u, t, d, n, A, lda, b, 1)
    r = opT @ b.astype(np.float64) - x.astype(np.float64)
    check(r, 0 * r, np.abs(opT) @ np.abs(b.astype(np.float64)), 2 * n, p, "trsv residual")


@pytest.mark.gpu
@pytest.mark.parametrize("p", "sd")
@pytest.mark.parametrize("side,u", [(LEFT, UP), (RIGHT, LO)])
def test_symm_syrk_syr2k_colmajor(colmajor, p, side, u):
    eb, g = colmajor, np.random.default_rng(5)
    m, n, k = 33, 27, 19
    ka = m if side == LEFT else n
    lda, ldb, ldc = ka + 2, m + 1, m + 3
    A = g.uniform(-1, 1, lda * ka).astype(DT[p])
    B = g.uniform(-1, 1, ldb * n).astype(DT[p])
    C = g.uniform(-1, 1, ldc * n).astype(DT[p])
    S = sym(cm(A.astype(np.float64), ka, ka, lda), u == UP)
    B64, C64 = cm(B.astype(np.float64), m, n, ldb), cm(C.astype(np.float64), m, n, ldc)
    prod, mprod = (S @ B64, np.abs(S) @ np.abs(B64)) if side == LEFT else (B64 @ S, np.abs(B64) @ np.abs(S))
    getattr(eb, f"exo_{p}symm")(COL, side, u, m, n, 1.5, A, lda, B, ldb, 0.5, C, ldc)
    check(cm(C, m, n, ldc), 1.5 * prod + 0.5 * C64, 1.5 * mprod + 0.5 * np.abs(C64), ka + 1, p, "symm")
    for t in (NT, TR):
        ar, ac = (n, k) if t == NT else (k, n)
        lda2 = ar + 1
        A2 = g.uniform(-1, 1, lda2 * ac).astype(DT[p])
        B2 = g.uniform(-1, 1, lda2 * ac).astype(DT[p])
        C2 = g.uniform(-1, 1, (n + 1) * n).astype(DT[p])
        a64, b64 = cm(A2.astype(np.float64), ar, ac, lda2), cm(B2.astype(np.float64), ar, ac, lda2)
        opA, opB = (a64, b64) if t == NT else (a64.T, b64.T)
        C0 = cm(C2.astype(np.float64), n, n, n + 1).copy()
        keep = np.triu(np.ones((n, n), bool)) if u == UP else np.tril(np.ones((n, n), bool))
        Cs = C2.copy()
        getattr(eb, f"exo_{p}syrk")(COL, u, t, n, k, 2.0, A2, lda2, 0.5, Cs, n + 1)
        ref = np.where(keep, 2.0 * opA @ opA.T + 0.5 * C0, C0)
        mag = np.where(keep, 2.0 * np.abs(opA) @ np.abs(opA.T) + 0.5 * np.abs(C0), np.abs(C0))
        check(cm(Cs, n, n, n + 1), ref, mag, k + 1, p, "syrk")
        Cs = C2.copy()
        getattr(eb, f"exo_{p}syr2k")(COL, u, t, n, k, 2.0, A2, lda2, B2, lda2, 0.5, Cs, n + 1)
        ref = np.where(keep, 2.0 * (opA @ opB.T + opB @ opA.T) + 0.5 * C0, C0)
        mag = np.where(keep, 2.0 * (np.abs(opA) @ np.abs(opB.T) + np.abs(opB) @ np.abs(opA.T)) + 0.5 * np.abs(C0),
                       np.abs(C0))
        check(cm(Cs, n, n, n + 1), ref, mag, 2 * k + 1, p, "syr2k")


@pytest.mark.gpu
@pytest.mark.parametrize("side,u,t,d", [(LEFT, UP, NT, NU), (LEFT, LO, TR, UN), (RIGHT, UP, TR, NU),
                                         (RIGHT, LO, NT, UN)])
def test_strmm_colmajor(colmajor, side, u, t, d):
    eb, g = colmajor, np.random.default_rng(6)
    m, n = 29, 22
    ka = m if side == LEFT else n
    lda, ldb = ka + 1, m + 2
    A = g.uniform(-1, 1, lda * ka).astype(np.float32)
    B = g.uniform(-1, 1, ldb * n).astype(np.float32)
    T = tri(cm(A.astype(np.float64), ka, ka, lda), u == UP, d == UN)
    opT = T if t == NT else T.T
    B64 = cm(B.astype(np.float64), m, n, ldb).copy()
    ref, mag = (opT @ B64, np.abs(opT) @ np.abs(B64)) if side == LEFT else (B64 @ opT, np.abs(B64) @ np.abs(opT))
    eb.exo_strmm(COL, side, u, t, d, m, n, 1.4, A, lda, B, ldb)
    check(cm(B, m, n, ldb), 1.4 * ref, 1.4 * mag, ka + 1, "s", "strmm")


@pytest.mark.gpu
def test_colmajor_rejected_by_default(cuda):
    import exoblas_gb300 as eb

    C = np.zeros(4, np.float32)
    with pytest.raises(eb.UnsupportedParameterException):
        eb.exo_sgemm(COL, NT, NT, 2, 2, 2, 1.0, C, 2, C, 2, 0.0, C.copy(), 2)


def band_cm(buf, n, k, lda, upper):
    """Dense n x n matrix from CBLAS column-major band storage: column j holds
    rows max(0, j-k)..j at buf[j*lda + k + i - j] (upper) or rows
    j..min(n-1, j+k) at buf[j*lda + i - j] (lower)."""
    A = np.zeros((n, n))
    for j in range(n):
        rows = range(max(0, j - k), j + 1) if upper else range(j, min(n, j + k + 1))
        for i in rows:
            A[i, j] = buf[j * lda + (k + i - j if upper else i - j)]
    return A


@pytest.mark.gpu
@pytest.mark.parametrize("p", "sd")
@pytest.mark.parametrize("u", [UP, LO])
def test_band_colmajor(colmajor, p, u):
    eb, g = colmajor, np.random.default_rng(6)
    n, k = 90, 7
    lda = k + 3
    a = (g.uniform(-1, 1, lda * n) / 100).astype(DT[p])
    for j in range(n):  # diagonal entries 2, as the reference's tbsv test
        a[j * lda + (k if u == UP else 0)] = 2
    B = band_cm(a.astype(np.float64), n, k, lda, u == UP)
    x = g.uniform(-1, 1, n).astype(DT[p])
    y = g.uniform(-1, 1, n).astype(DT[p])
    x64, y64 = x.astype(np.float64), y.astype(np.float64)
    # sbmv: the stored triangle defines the symmetric band matrix
    S = B + B.T - np.diag(np.diag(B))
    yy = y.copy()
    getattr(eb, f"exo_{p}sbmv")(COL, u, n, k, 1.3, a, lda, x, 1, 0.4, yy, 1)
    check(yy, 1.3 * S @ x64 + 0.4 * y64, 1.3 * np.abs(S) @ np.abs(x64) + 0.4 * np.abs(y64), 2 * k + 2, p, "sbmv")
    for t in (NT, TR):
        for d in (NU, UN):
            T = B.copy()
            if d == UN:
                np.fill_diagonal(T, 1.0)
            opT = T if t == NT else T.T
            xm = x.copy()
            getattr(eb, f"exo_{p}tbmv")(COL, u, t, d, n, k, a, lda, xm, 1)
            check(xm, opT @ x64, np.abs(opT) @ np.abs(x64), k + 2, p, f"tbmv t={t} d={d}")
            b = x.copy()
            getattr(eb, f"exo_{p}tbsv")(COL, u, t, d, n, k, a, lda, b, 1)
            b64 = b.astype(np.float64)
            r = opT @ b64 - x64
            check(r, 0 * r, np.abs(opT) @ np.abs(b64), 2 * (k + 1), p, f"tbsv residual t={t} d={d}")
