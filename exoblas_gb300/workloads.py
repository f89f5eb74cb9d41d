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
