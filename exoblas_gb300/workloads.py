"""Seeded synthetic workloads with the shapes of the benchmark configurations
(device-resident torch tensors; used by bench.py and the tests).

batch_config(): 4096 independent instances of sgemm NN / dgemv N / strsv
(lower, no-trans, non-unit), the op drawn uniformly per instance and m, n, k
log-uniform in [16, 2048] from seed 7; entries uniform[-1, 1); the strsv
matrices have diagonal 1 + uniform[0, 1) and off-diagonal uniform[-1, 1)/n
(well conditioned: with unscaled off-diagonals the solution grows
exponentially with n and overflows FP32).
"""
from __future__ import annotations

import math

import numpy as np

OPS = ("sgemm", "dgemv", "strsv")


def log_uniform(rng, lo, hi, size=None):
    return np.exp(rng.uniform(math.log(lo), math.log(hi + 1), size)).astype(np.int64).clip(lo, hi)


def batch_shapes(count=4096, seed=7, lo=16, hi=2048):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        op = OPS[int(rng.integers(0, 3))]
        m, n, k = (int(v) for v in log_uniform(rng, lo, hi, 3))
        out.append((op, m, n, k))
    return out


class Arena:
    """One device buffer per dtype, carved into operands (few allocations)."""

    def __init__(self, torch, device, nfloat, ndouble, seed=7):
        self.torch = torch
        g = torch.Generator(device=device).manual_seed(seed)
        self.f = torch.rand(max(nfloat, 1), device=device, generator=g, dtype=torch.float32).mul_(2).sub_(1)
        self.d = torch.rand(max(ndouble, 1), device=device, generator=g, dtype=torch.float64).mul_(2).sub_(1)
        self.of = 0
        self.od = 0

    def take(self, n, double=False):
        # 64-element alignment keeps every operand 256-byte aligned
        n = int(n)
        if double:
            t = self.d[self.od:self.od + n]
            self.od += (n + 63) // 64 * 64
        else:
            t = self.f[self.of:self.of + n]
            self.of += (n + 63) // 64 * 64
        return t


def batch_config(torch, device="cuda", count=4096, seed=7, lo=16, hi=2048):
    """Returns (ops, shapes, arena, views): BatchOp list plus the tensors."""
    from .batch import BatchOp

    shapes = batch_shapes(count, seed, lo, hi)
    nf = nd = 0
    for op, m, n, k in shapes:
        if op == "sgemm":
            nf += (m * k + k * n + m * n) + 3 * 64
        elif op == "dgemv":
            nd += (m * n + n + m) + 3 * 64
        else:
            nf += (m * m + m) + 2 * 64
    ar = Arena(torch, device, nf, nd, seed)
    ops, views = [], []
    for op, m, n, k in shapes:
        if op == "sgemm":
            A, B, Cm = ar.take(m * k), ar.take(k * n), ar.take(m * n)
            ops.append(BatchOp.sgemm(111, 111, m, n, k, 1.0, A, k, B, n, 0.5, Cm, n))
            views.append((op, (m, n, k), (A, B, Cm)))
        elif op == "dgemv":
            A, x, y = ar.take(m * n, True), ar.take(n, True), ar.take(m, True)
            ops.append(BatchOp.dgemv(111, m, n, 1.0, A, n, x, 1, 0.5, y, 1))
            views.append((op, (m, n), (A, x, y)))
        else:
            A, x = ar.take(m * m), ar.take(m)
            M = A.view(m, m)
            M.div_(m)
            M.diagonal().copy_(1.0 + torch.rand(m, device=device, generator=torch.Generator(device=device).manual_seed(len(ops))))
            ops.append(BatchOp.strsv(122, 111, 131, m, A, m, x, 1))
            views.append((op, (m,), (A, x)))
    return ops, shapes, ar, views


# ------------------------------------------------------------------ serving --
SERVE_MIX = (("gemm", 0.60), ("gemv", 0.25), ("trsv", 0.10), ("syrk", 0.05))


def serve_stream(count, rate=20000.0, seed_arrivals=11, seed_ops=12, lo=32, hi=8192, fp32_share=0.7):
    """A Poisson request stream: exponential inter-arrival gaps of mean
    1/rate (seed_arrivals); per request the op from SERVE_MIX, precision
    single with probability fp32_share, and every dimension log-uniform in
    [lo, hi] (seed_ops).  Returns [(offset_s, op, precision, m, n, k)]."""
    ga = np.random.default_rng(seed_arrivals)
    go = np.random.default_rng(seed_ops)
    t = np.cumsum(ga.exponential(1.0 / rate, count))
    t -= t[0]
    names = [m[0] for m in SERVE_MIX]
    probs = np.array([m[1] for m in SERVE_MIX])
    ops = go.choice(len(names), size=count, p=probs / probs.sum())
    prec = np.where(go.uniform(size=count) < fp32_share, 1, 2)
    dims = log_uniform(go, lo, hi, (count, 3))
    return [(float(t[i]), names[ops[i]], int(prec[i]), int(dims[i, 0]), int(dims[i, 1]), int(dims[i, 2]))
            for i in range(count)]


class ServeOperands:
    """Device-resident operands for a request stream.

    Inputs (A, B, x) are read-only windows at seeded 256-byte aligned offsets
    of one uniform[-1, 1) buffer per precision (in_elems elements); outputs
    (C, y, and trsv's x, solved in place) are carved in arrival order from a
    ring per precision (out_elems elements, uniform[-1, 1) at start), so
    requests close together in the stream never share an output.  trsv reads
    the leading n x n block of one hi x hi lower-triangular matrix per
    precision with off-diagonal uniform[-1, 1)/hi and diagonal
    1 + uniform[0, 1) (well conditioned at every n)."""

    def __init__(self, torch, device="cuda", in_elems=(1 << 30, 1 << 29), out_elems=(1 << 30, 1 << 29), hi=8192,
                 seed=12):
        self.torch = torch
        g = torch.Generator(device=device).manual_seed(seed)
        self.inp = {}
        self.out = {}
        self.tri = {}
        for p, dt, ni, no in ((1, torch.float32, in_elems[0], out_elems[0]), (2, torch.float64, in_elems[1],
                                                                                   out_elems[1])):
            self.inp[p] = torch.rand(ni, device=device, generator=g, dtype=dt).mul_(2).sub_(1)
            self.out[p] = torch.rand(no, device=device, generator=g, dtype=dt).mul_(2).sub_(1)
            T = torch.rand(hi, hi, device=device, generator=g, dtype=dt).mul_(2).sub_(1).div_(hi)
            T.diagonal().copy_(1.0 + torch.rand(hi, device=device, generator=g, dtype=dt))
            self.tri[p] = T
        self.hi = hi
        self.rng = np.random.default_rng(seed)
        self.ring = {1: 0, 2: 0}

    def _in(self, p, n):
        buf = self.inp[p]
        span = buf.numel() - n
        off = int(self.rng.integers(0, max(span, 0) // 64 + 1)) * 64
        return buf[off:off + n]

    def _out(self, p, n):
        buf = self.out[p]
        if self.ring[p] + n > buf.numel():
            self.ring[p] = 0
        o = self.ring[p]
        self.ring[p] += (n + 63) // 64 * 64
        return buf[o:o + n]

    def request(self, op, p, m, n, k):
        """(Request, views) for one stream entry: gemm NN C[m,n] = A[m,k] B[k,n]
        + 0.5 C; gemv N y[m] = A[m,n] x + 0.5 y; trsv lower / no-trans /
        non-unit of order m; syrk lower / no-trans C[m,m] = A[m,k] A^T + 0.5 C."""
        from . import serve

        if op == "gemm":
            A, B, Cm = self._in(p, m * k), self._in(p, k * n), self._out(p, m * n)
            r = serve.request(serve.GEMM, p, (111, 111), m, n, k, 1.0, 0.5, A, k, B, n, Cm, n)
            return r, (A, B, Cm)
        if op == "gemv":
            A, x, y = self._in(p, m * n), self._in(p, n), self._out(p, m)
            r = serve.request(serve.GEMV, p, (111,), m, n, 0, 1.0, 0.5, A, n, x, 1, y, 1)
            return r, (A, x, y)
        if op == "trsv":
            x = self._out(p, m)
            r = serve.request(serve.TRSV, p, (122, 111, 131), m, 0, 0, 1.0, 0.0, self.tri[p], self.hi, None, 0, x, 1)
            return r, (self.tri[p], x)
        A, Cm = self._in(p, m * k), self._out(p, m * m)
        r = serve.request(serve.SYRK, p, (122, 111), m, 0, k, 1.0, 0.5, A, k, None, 0, Cm, m)
        return r, (A, Cm)


def request_work(op, m, n, k, p):
    """(flops, bytes) of one request: 2mnk for gemm, m(m+1)k for syrk; gemv
    and trsv by the bytes of A and the vectors they stream."""
    es = 4 if p == 1 else 8
    if op == "gemm":
        return 2.0 * m * n * k, 0.0
    if op == "syrk":
        return float(m) * (m + 1) * k, 0.0
    if op == "gemv":
        return 2.0 * m * n, float(m * n + n + 2 * m) * es
    return float(m) * m, float(m * (m + 1) // 2 + 2 * m) * es
