"""Parameter grids of the reference's correctness tests, as seeded Cases.

Each generator follows test/level*/<op>/correctness.cpp of the reference
(grids cited per function) and yields Cases whose argument lists match the
exo_<p><op> C signatures.
"""
from __future__ import annotations

import itertools
import zlib

import numpy as np

from common import DT, LEFT, LO, NT, NU, RIGHT, ROW, TR, UN, UP, Case, buf, mat, rng


def _seed(*key):
    return zlib.crc32(repr(key).encode())


# ------------------------------------------------------------------ level 1 --

L1_N = [2, 321, 1000]  # every test/level1/*/correctness.cpp uses N{2, 321, 1000}


def asum_cases(p):  # test/level1/asum/correctness.cpp:30-31
    for n, inc in itertools.product(L1_N, [1, 3]):
        g = rng(_seed("asum", p, n, inc))
        x = buf(g, n, inc, DT[p])
        yield Case(p + "asum", [n, x, inc], [], scalar=True, nred=n, label=f"n={n} inc={inc}")


def axpy_cases(p):  # test/level1/axpy/correctness.cpp:30-32
    params = [(a, 1, 1) for a in (1.2, 0.0, 1.0)] + [(1.2, 2, 2), (1.2, -2, 3), (0.7, 1, -2)]
    for n, (alpha, ix, iy) in itertools.product(L1_N, params):
        g = rng(_seed("axpy", p, n, alpha, ix, iy))
        x, y = buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
        yield Case(p + "axpy", [n, alpha, x, ix, y, iy], [4], nred=2, label=f"n={n} a={alpha} inc=({ix},{iy})")


def dot_cases(p):  # test/level1/dot/correctness.cpp:30-31
    for n, (ix, iy) in itertools.product(L1_N, [(1, 1), (3, 3), (-2, 1)]):
        g = rng(_seed("dot", p, n, ix, iy))
        x, y = buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
        yield Case(p + "dot", [n, x, ix, y, iy], [], scalar=True, nred=n, label=f"n={n} inc=({ix},{iy})")


def dsdot_cases():  # test/level1/dsdot/correctness.cpp:25-26
    for n, (ix, iy) in itertools.product(L1_N, [(1, 1), (2, 2), (-2, -4)]):
        g = rng(_seed("dsdot", n, ix, iy))
        x, y = buf(g, n, ix, np.float32), buf(g, n, iy, np.float32)
        yield Case("dsdot", [n, x, ix, y, iy], [], scalar=True, nred=n, label=f"n={n} inc=({ix},{iy})")


def sdsdot_cases():  # test/level1/sdsdot/correctness.cpp:25-26
    for n, (ix, iy) in itertools.product(L1_N, [(1, 1), (2, 2), (-2, -4)]):
        g = rng(_seed("sdsdot", n, ix, iy))
        x, y = buf(g, n, ix, np.float32), buf(g, n, iy, np.float32)
        yield Case("sdsdot", [n, 0.75, x, ix, y, iy], [], scalar=True, nred=n, label=f"n={n} inc=({ix},{iy})")


def copy_cases(p):  # test/level1/copy/correctness.cpp:30-31
    for n, (ix, iy) in itertools.product(L1_N, [(1, 1), (2, 2), (-3, 2)]):
        g = rng(_seed("copy", p, n, ix, iy))
        x, y = buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
        yield Case(p + "copy", [n, x, ix, y, iy], [3], exact=True, label=f"n={n} inc=({ix},{iy})")


def swap_cases(p):  # test/level1/swap/correctness.cpp:30-31
    for n, (ix, iy) in itertools.product(L1_N, [(1, 1), (2, 2), (2, -3)]):
        g = rng(_seed("swap", p, n, ix, iy))
        x, y = buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
        yield Case(p + "swap", [n, x, ix, y, iy], [1, 3], exact=True, label=f"n={n} inc=({ix},{iy})")


def scal_cases(p):  # test/level1/scal/correctness.cpp:28-30
    params = [(a, 1) for a in (0.0, 1.0, 2.0, -1.0)] + [(1.0, 4), (2.0, 4), (0.0, 4), (2.0, -1)]
    for n, (alpha, inc) in itertools.product(L1_N, params):
        g = rng(_seed("scal", p, n, alpha, inc))
        x = buf(g, n, inc, DT[p])
        exact = alpha in (0.0, 1.0, -1.0) or inc < 0
        yield Case(p + "scal", [n, alpha, x, inc], [2], nred=1, exact=exact, label=f"n={n} a={alpha} inc={inc}")


def rot_cases(p):  # test/level1/rot/correctness.cpp:29-31
    params = [(1, 1, 2.0, 3.0), (2, 2, 1.0, 2.0), (-1, 2, 0.6, 0.8)]
    for n, (ix, iy, c, s) in itertools.product(L1_N, params):
        g = rng(_seed("rot", p, n, ix, iy, c, s))
        x, y = buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
        yield Case(p + "rot", [n, x, ix, y, iy, c, s], [1, 3], nred=2, label=f"n={n} inc=({ix},{iy})")


def rotm_cases(p):  # test/level1/rotm/correctness.cpp:17-35 (flags -2, -1, 0, 1)
    for n, (ix, iy), flag in itertools.product(L1_N, [(1, 1), (2, 2), (-2, 1)], [-2.0, -1.0, 0.0, 1.0]):
        g = rng(_seed("rotm", p, n, ix, iy, flag))
        x, y = buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
        P = np.array([flag, 1.2, 2.2, 3.2, 4.2], DT[p])
        yield Case(p + "rotm", [n, x, ix, y, iy, P], [1, 3], nred=2, exact=(flag == -2.0),
                   label=f"n={n} inc=({ix},{iy}) flag={flag}")


def level1_cases():
    for p in "sd":
        yield from asum_cases(p)
        yield from axpy_cases(p)
        yield from dot_cases(p)
        yield from copy_cases(p)
        yield from swap_cases(p)
        yield from scal_cases(p)
        yield from rot_cases(p)
        yield from rotm_cases(p)
    yield from dsdot_cases()
    yield from sdsdot_cases()


# ------------------------------------------------------------------ level 2 --


def gemv_cases(p, Ns=(3, 41, 80, 101, 141, 1024), Ms=(77, 103, 500)):
    """test/level2/gemv/correctness.cpp:46-76"""
    for t, n, m, ldd, ix, iy in itertools.product((NT, TR), Ns, Ms, (0, 5), (1, 2), (1, -3)):
        g = rng(_seed("gemv", p, t, n, m, ldd, ix, iy))
        lda = n + ldd
        A = mat(g, m, lda, DT[p])
        sx, sy = (n, m) if t == NT else (m, n)
        x, y = buf(g, sx, ix, DT[p]), buf(g, sy, iy, DT[p])
        yield Case(p + "gemv", [ROW, t, m, n, 2.4, A, lda, x, ix, 2.4, y, iy], [10], nred=sx + 1,
                   label=f"t={t} m={m} n={n} lda={lda} inc=({ix},{iy})")


def ger_cases(p, Ms=(77, 103, 500), Ns=(41, 80, 101, 1024)):
    """test/level2/ger/correctness.cpp:35-42"""
    for m, n, ldd, ix, iy in itertools.product(Ms, Ns, (0, 5), (1, 2), (1, -3)):
        g = rng(_seed("ger", p, m, n, ldd, ix, iy))
        lda = n + ldd
        A = mat(g, m, lda, DT[p])
        x, y = buf(g, m, ix, DT[p]), buf(g, n, iy, DT[p])
        yield Case(p + "ger", [ROW, m, n, 2.4, x, ix, y, iy, A, lda], [8], nred=2,
                   label=f"m={m} n={n} lda={lda} inc=({ix},{iy})")


def symv_cases(p, Ns=(2, 100, 321)):
    """test/level2/symv/correctness.cpp:37-44"""
    for u, n, alpha, ldd, ix, beta, iy in itertools.product((UP, LO), Ns, (1.0, 2.4), (0, 3), (1, 3), (0.0, 2.4), (1, -2)):
        g = rng(_seed("symv", p, u, n, alpha, ldd, ix, beta, iy))
        lda = n + ldd
        A = mat(g, n, lda, DT[p])
        x, y = buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
        yield Case(p + "symv", [ROW, u, n, alpha, A, lda, x, ix, beta, y, iy], [9], nred=n + 1,
                   label=f"u={u} n={n} a={alpha} b={beta} lda={lda} inc=({ix},{iy})")


def syr_cases(p, Ns=(2, 100, 321, 1115)):
    """test/level2/syr/correctness.cpp:32-37"""
    for u, n, ix, ldd in itertools.product((UP, LO), Ns, (1, 2, -1), (0, 5)):
        g = rng(_seed("syr", p, u, n, ix, ldd))
        lda = n + ldd
        A = mat(g, n, lda, DT[p])
        x = buf(g, n, ix, DT[p])
        yield Case(p + "syr", [ROW, u, n, 1.2, x, ix, A, lda], [6], nred=2, label=f"u={u} n={n} lda={lda} inc={ix}")


def syr2_cases(p, Ns=(2, 100, 321)):
    """test/level2/syr2/correctness.cpp:35-41"""
    for u, n, ix, iy, ldd in itertools.product((UP, LO), Ns, (1, 2), (1, -3), (0, 5)):
        g = rng(_seed("syr2", p, u, n, ix, iy, ldd))
        lda = n + ldd
        A = mat(g, n, lda, DT[p])
        x, y = buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
        yield Case(p + "syr2", [ROW, u, n, 1.2, x, ix, y, iy, A, lda], [8], nred=3,
                   label=f"u={u} n={n} lda={lda} inc=({ix},{iy})")


def trmv_cases(p, Ns=(2, 100, 321)):
    """test/level2/trmv/correctness.cpp:33-39"""
    for u, t, d, n, ix, ldd in itertools.product((UP, LO), (NT, TR), (UN, NU), Ns, (1, 2, -2), (0, 5)):
        g = rng(_seed("trmv", p, u, t, d, n, ix, ldd))
        lda = n + ldd
        A = mat(g, n, lda, DT[p])
        x = buf(g, n, ix, DT[p])
        yield Case(p + "trmv", [ROW, u, t, d, n, A, lda, x, ix], [7], nred=n + 1,
                   label=f"u={u} t={t} d={d} n={n} lda={lda} inc={ix}")


def trsv_cases(p, Ns=(2, 100, 321), fixture=False, incs=(1, 2, -2), ldds=(0, 5)):
    """test/level2/trsv/correctness.cpp:42-58.  fixture=True reproduces the
    reference's deterministic inputs (A[i*lda+j] = 2 + j/N in integer
    arithmetic, i.e. all 2.0; X[i] = i, :20-25); otherwise A is
    well-conditioned (off-diagonal uniform[-1,1)/n, diagonal 1 + uniform[0,1))."""
    for u, t, d, n, ix, ldd in itertools.product((UP, LO), (NT, TR), (UN, NU), Ns, incs, ldds):
        lda = n + ldd
        if fixture:
            if ix < 0:
                continue
            A = np.full(n * lda, 2.0 + 0 // n, DT[p])
            x = np.arange(1 + (n - 1) * abs(ix), dtype=DT[p])
        else:
            g = rng(_seed("trsv", p, u, t, d, n, ix, ldd))
            A = (g.uniform(-1.0, 1.0, n * lda) / n).reshape(n, lda)
            A[np.arange(n), np.arange(n)] = 1.0 + g.uniform(0.0, 1.0, n)
            A = A.astype(DT[p]).ravel()
            x = buf(g, n, ix, DT[p])
        yield Case(p + "trsv", [ROW, u, t, d, n, A, lda, x, ix], [7], nred=n + 1,
                   label=f"u={u} t={t} d={d} n={n} lda={lda} inc={ix}{' fixture' if fixture else ''}")


# ------------------------------------------------------------------ level 3 --

L3_DIMS = (1, 7, 32, 64, 257)  # gemm/symm/syrk correctness.cpp dims


def gemm_cases(p, dims=L3_DIMS, ldds=(0, 5)):
    """test/level3/gemm/correctness.cpp:45-63 (alpha 13, beta 18)"""
    for m, n, k, ta, tb, ldd in itertools.product(dims, dims, dims, (NT, TR), (NT, TR), ldds):
        g = rng(_seed("gemm", p, m, n, k, ta, tb, ldd))
        ar, ac = (m, k) if ta == NT else (k, m)
        br, bc = (k, n) if tb == NT else (n, k)
        lda, ldb, ldc = ac + ldd, bc + ldd, n + ldd
        A, B, C = mat(g, ar, lda, DT[p]), mat(g, br, ldb, DT[p]), mat(g, m, ldc, DT[p])
        yield Case(p + "gemm", [ROW, ta, tb, m, n, k, 13.0, A, lda, B, ldb, 18.0, C, ldc], [12], nred=k + 1,
                   label=f"m={m} n={n} k={k} t=({ta},{tb}) ldd={ldd}")


def symm_cases(p, dims=L3_DIMS, ldds=(0, 5)):
    """test/level3/symm/correctness.cpp:43-62"""
    for side, u, m, n, ldd in itertools.product((LEFT, RIGHT), (LO, UP), dims, dims, ldds):
        g = rng(_seed("symm", p, side, u, m, n, ldd))
        ka = m if side == LEFT else n
        lda, ldb, ldc = ka + ldd, n + ldd, n + ldd
        A, B, C = mat(g, ka, lda, DT[p]), mat(g, m, ldb, DT[p]), mat(g, m, ldc, DT[p])
        yield Case(p + "symm", [ROW, side, u, m, n, 13.0, A, lda, B, ldb, 18.0, C, ldc], [11], nred=ka + 1,
                   label=f"side={side} u={u} m={m} n={n} ldd={ldd}")


def syrk_cases(p, dims=L3_DIMS, ldds=(0, 5)):
    """test/level3/syrk/correctness.cpp:39-55"""
    for n, k, t, u, ldd in itertools.product(dims, dims, (NT, TR), (LO, UP), ldds):
        g = rng(_seed("syrk", p, n, k, t, u, ldd))
        ar, ac = (n, k) if t == NT else (k, n)
        lda, ldc = ac + ldd, n + ldd
        A, C = mat(g, ar, lda, DT[p]), mat(g, n, ldc, DT[p])
        yield Case(p + "syrk", [ROW, u, t, n, k, 13.0, A, lda, 18.0, C, ldc], [9], nred=k + 1,
                   label=f"n={n} k={k} t={t} u={u} ldd={ldd}")


def syr2k_cases(p, dims=L3_DIMS, ldds=(0, 5)):
    """test/level3/syr2k/correctness.cpp:13-62 (alpha 13, beta 18)"""
    for u, n, k, t, da, db, dc in itertools.product((LO, UP), dims, dims, (NT, TR), ldds, ldds, ldds):
        g = rng(_seed("syr2k", p, u, n, k, t, da, db, dc))
        ar, ac = (n, k) if t == NT else (k, n)
        lda, ldb, ldc = ac + da, ac + db, n + dc
        A, B, C = mat(g, ar, lda, DT[p]), mat(g, ar, ldb, DT[p]), mat(g, n, ldc, DT[p])
        yield Case(p + "syr2k", [ROW, u, t, n, k, 13.0, A, lda, B, ldb, 18.0, C, ldc], [11], nred=2 * k + 1,
                   label=f"u={u} n={n} k={k} t={t} lda={lda} ldb={ldb} ldc={ldc}")


def trmm_cases(Ms=(4, 101, 321), Ns=(8, 15, 564), alphas=(0.0, 1.0, 1.4), ldds=(0, 5)):
    """test/level3/strmm/correctness.cpp:11-80 (float only, Side Left; A and
    B are AlignedBuffer(K * lda) / AlignedBuffer(M * ldb) of uniform[-1, 1))"""
    for m, n, u, t, d, al, da, db in itertools.product(Ms, Ns, (UP, LO), (NT, TR), (NU, UN), alphas, ldds, ldds):
        g = rng(_seed("trmm", m, n, u, t, d, al, da, db))
        lda, ldb = m + da, n + db
        A, B = mat(g, m, lda, np.float32), mat(g, m, ldb, np.float32)
        yield Case("strmm", [ROW, LEFT, u, t, d, m, n, al, A, lda, B, ldb], [10], nred=m + 1,
                   label=f"m={m} n={n} u={u} t={t} d={d} alpha={al} lda={lda} ldb={ldb}")


# ------------------------------------------------------------ banded level 2 --

def gbmv_cases(p, sizes=((2, 2, 1, 1), (15, 20, 0, 5), (256, 256, 255, 255)), incs=((1, 1),)):
    """test/level2/sgbmv/correctness.cpp:36-50 (alpha = beta = 1.2, lda = KL + KU + 1)"""
    for (m, n, kl, ku), (ix, iy) in itertools.product(sizes, incs):
        g = rng(_seed("gbmv", p, m, n, kl, ku, ix, iy))
        lda = kl + ku + 1
        A, x, y = mat(g, m, lda, DT[p]), buf(g, n, ix, DT[p]), buf(g, m, iy, DT[p])
        yield Case(p + "gbmv", [m, n, kl, ku, 1.2, A, lda, x, ix, 1.2, y, iy], [10], nred=kl + ku + 2,
                   label=f"m={m} n={n} kl={kl} ku={ku} incx={ix} incy={iy}", extra={"tol": 1e-3})


def sbmv_cases(p, Ns=(2, 100, 321), Ks=(0, 1, 50)):
    """test/level2/ssbmv/correctness.cpp:39-70 (alpha 2.4; beta 0, 1; incX 1, 3;
    incY 1, -2; lda = K + 1 + {0, 3}, plus K = N - 1 with lda = N + {0, 3})"""
    for u, n, ldd, ix, be, iy in itertools.product((UP, LO), Ns, (0, 3), (1, 3), (0.0, 1.0), (1, -2)):
        for k, lda in [(k, k + 1 + ldd) for k in Ks if k <= n - 1] + [(n - 1, n + ldd)]:
            g = rng(_seed("sbmv", p, u, n, k, ldd, ix, be, iy))
            A, x, y = mat(g, n, lda, DT[p]), buf(g, n, ix, DT[p]), buf(g, n, iy, DT[p])
            yield Case(p + "sbmv", [ROW, u, n, k, 2.4, A, lda, x, ix, be, y, iy], [10], nred=2 * k + 2,
                       label=f"u={u} n={n} k={k} lda={lda} incx={ix} beta={be} incy={iy}")


def tbmv_cases(p, Ns=(2, 100, 321), Ks=(0, 1, 6)):
    """test/level2/stbmv/correctness.cpp:37-64 (lda = K + 1 + {0, 3}, incX 1, 3,
    plus K = N - 1 with lda = N + {0, 3})"""
    for n, u, t, d, ldd, ix in itertools.product(Ns, (UP, LO), (NT, TR), (NU, UN), (0, 3), (1, 3)):
        for k, lda in [(k, k + 1 + ldd) for k in Ks if k <= n - 1] + [(n - 1, n + ldd)]:
            g = rng(_seed("tbmv", p, n, u, t, d, k, ldd, ix))
            A, x = mat(g, n, lda, DT[p]), buf(g, n, ix, DT[p])
            yield Case(p + "tbmv", [ROW, u, t, d, n, k, A, lda, x, ix], [8], nred=k + 1,
                       label=f"n={n} u={u} t={t} d={d} k={k} lda={lda} incx={ix}")


def tbsv_cases(p, Ns=(2, 100, 321), Ks=(0, 1, 2, 10, 60)):
    """test/level2/stbsv/correctness.cpp:11-75: A uniform[-1, 1) / 1000 with the
    diagonal entries set to 2; lda = K + 1 (the reference's loop also repeats
    K = N - 1 with lda = N + {0, 3} per K)"""
    for n, u, t, d, ldd, ix in itertools.product(Ns, (UP, LO), (NT, TR), (UN, NU), (0, 3), (1, 3)):
        for k, lda in [(k, k + 1 + ldd) for k in Ks if k <= n - 1] + [(n - 1, n + ldd)]:
            g = rng(_seed("tbsv", p, n, u, t, d, k, ldd, ix))
            A = (g.uniform(-1.0, 1.0, n * lda) / 1000).astype(DT[p])
            A.reshape(n, lda)[:, 0 if u == UP else k] = 2
            x = buf(g, n, ix, DT[p])
            yield Case(p + "tbsv", [ROW, u, t, d, n, k, A, lda, x, ix], [8], nred=k + 1,
                       label=f"n={n} u={u} t={t} d={d} k={k} lda={lda} incx={ix}")


# ---------------------------------------------------------------- nrm2, iamax --

def nrm2_cases(p, Ns=(1, 2, 7, 100, 1000, 20000), incs=(1, 3, -1, 0), scales=(1.0, 1e200, 1e-200)):
    """nrm2 has no reference test (README.md:15); sizes and increments follow
    the level-1 grids, plus FP64 magnitudes whose squares overflow or
    underflow, and non-positive increments (result 0)."""
    for n, inc, sc in itertools.product(Ns, incs, scales):
        if p == "s" and sc != 1.0:
            sc = 1e30 if sc > 1 else 1e-30  # FP32 magnitudes whose squares overflow / underflow
        g = rng(_seed("nrm2", p, n, inc, sc))
        x = (buf(g, n, max(abs(inc), 1), np.float64) * sc).astype(DT[p])
        yield Case(p + "nrm2", [n, x, inc], [], scalar=True, nred=n, label=f"n={n} inc={inc} scale={sc:g}")


def iamax_cases(p, Ns=(1, 2, 7, 100, 1000, 20000), incs=(1, 3, -1, 0)):
    """i?amax: first index of the largest magnitude; ties planted so the
    first-index rule is exercised."""
    for n, inc, tie in itertools.product(Ns, incs, (False, True)):
        g = rng(_seed("iamax", p, n, inc, tie))
        x = buf(g, n, max(abs(inc), 1), DT[p])
        if tie and n > 2:
            step = max(abs(inc), 1)
            hi = DT[p](1.5)
            for pos in sorted(g.choice(n, 3, replace=False)):
                x[pos * step] = hi if pos % 2 else -hi
        yield Case(p[0] if False else ("i" + p + "amax"), [n, x, inc], [], scalar=True, exact=True, nred=n,
                   label=f"n={n} inc={inc} tie={tie}")

