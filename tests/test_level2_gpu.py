"""Level-2 parity on the GPU (grids of test/level2/*/correctness.cpp)."""
import numpy as np
import pytest

from cases import gemv_cases, ger_cases, symv_cases, syr2_cases, syr_cases, trmv_cases, trsv_cases
from common import EPS, assert_rel1pct, check_case, run_gpu, run_oracle, trsv_residual_ok

GENERAL = (
    [c for p in "sd" for c in gemv_cases(p)]
    + [c for p in "sd" for c in ger_cases(p)]
    + [c for p in "sd" for c in symv_cases(p)]
    + [c for p in "sd" for c in syr_cases(p)]
    + [c for p in "sd" for c in syr2_cases(p)]
    + [c for p in "sd" for c in trmv_cases(p)]
)


@pytest.mark.gpu
@pytest.mark.parametrize("case", GENERAL, ids=lambda c: f"{c.op}-{c.label}")
def test_level2_host_pointers(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", GENERAL[::7], ids=lambda c: f"{c.op}-{c.label}")
def test_level2_device_pointers(cuda, case):
    r, a = run_gpu(case, device=True)
    check_case(case, r, a)


TRSV = [c for p in "sd" for c in trsv_cases(p)] + [c for p in "sd" for c in trsv_cases(p, fixture=True)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", TRSV, ids=lambda c: f"{c.op}-{c.label}")
def test_trsv(cuda, case):
    r, a = run_gpu(case)
    o_r, o_a = run_oracle(case)
    assert_rel1pct(a[7], o_a[7], f"{case}")  # the reference's own check
    trsv_residual_ok(case, a[7])


@pytest.mark.gpu
def test_trsv_device_pointers(cuda):
    for case in [c for c in trsv_cases("d", Ns=(321,)) if c.args[8] == 1][:8]:
        r, a = run_gpu(case, device=True)
        trsv_residual_ok(case, a[7])


@pytest.mark.gpu
def test_sgemv_full_size_properties(cuda):
    """sgemv N and T at M = N = 16384: against a torch FP64 matvec within the
    componentwise bound (c = 4)."""
    import exoblas_gb300 as eb

    torch = cuda
    gen = torch.Generator(device="cuda").manual_seed(0)
    n = 16384
    A = torch.rand(n, n, device="cuda", generator=gen) * 2 - 1
    x = torch.rand(n, device="cuda", generator=gen) * 2 - 1
    y0 = torch.rand(n, device="cuda", generator=gen) * 2 - 1
    for t, op in ((111, A), (112, A.t())):
        y = y0.clone()
        eb.exo_sgemv(101, t, n, n, 1.5, A, n, x, 1, 0.5, y, 1)
        ref = 1.5 * (op.double() @ x.double()) + 0.5 * y0.double()
        mag = 1.5 * (op.double().abs() @ x.double().abs()) + 0.5 * y0.double().abs()
        err = (y.double() - ref).abs()
        assert torch.all(err <= 4 * n * EPS["s"] * mag), float((err / mag).max())


@pytest.mark.gpu
def test_dtrsv_full_size_dd(cuda):
    """dtrsv lower / no-trans / non-unit at n = 8192 with the benchmark's
    well-conditioned matrix, against the double-double oracle."""
    import exoblas_gb300 as eb
    import oracle

    n = 8192
    g = np.random.default_rng(0)
    A = g.uniform(-1, 1, (n, n)) / n
    A[np.arange(n), np.arange(n)] = 1.0 + g.uniform(0, 1, n)
    A = np.tril(A)
    b = g.uniform(-1, 1, n)
    x = b.copy()
    eb.exo_dtrsv(101, 122, 111, 131, n, A, n, x, 1)
    xr = b.copy()
    lo = np.zeros(n)
    oracle.call("dd_trsv", 122, 0, 131, n, A, n, xr, lo)
    fwd = np.abs(x - xr) / np.maximum(np.abs(xr), 1e-300)
    assert fwd.max() <= 64 * n * EPS["d"], fwd.max()


CLUSTER = [c for p in "sd" for c in trsv_cases(p, Ns=(1000, 2049, 4160), incs=(1,), ldds=(0,))]


@pytest.mark.gpu
@pytest.mark.parametrize("case", CLUSTER, ids=lambda c: f"{c.op}-{c.label}")
def test_trsv_clustered_sizes(cuda, case):
    """Sizes that take the clustered solver (unit stride, n >= 192), all
    Uplo x Trans x Diag combinations, with the residual bound."""
    r, a = run_gpu(case)
    o_r, o_a = run_oracle(case)
    assert_rel1pct(a[7], o_a[7], f"{case}")
    trsv_residual_ok(case, a[7])


@pytest.mark.gpu
def test_matrices_past_int32_elements(cuda):
    """n = 46341, so n * n > 2^31 elements (8.6 GB of FP32): gemv N / T and
    symv with A = ones and x = ones give y = n exactly (integer partial sums
    below 2^24 are exact in FP32), which exercises every row and column and
    the 64-bit element offsets."""
    import torch

    import exoblas_gb300 as eb

    n = 46341
    A = torch.ones((n, n), dtype=torch.float32, device="cuda")
    x = torch.ones(n, dtype=torch.float32, device="cuda")
    for trans in (111, 112):
        y = torch.zeros(n, dtype=torch.float32, device="cuda")
        eb.exo_sgemv(101, trans, n, n, 1.0, A, n, x, 1, 0.0, y, 1)
        torch.cuda.synchronize()
        assert bool((y == float(n)).all()), trans
    for uplo in (121, 122):
        y = torch.zeros(n, dtype=torch.float32, device="cuda")
        eb.exo_ssymv(101, uplo, n, 1.0, A, n, x, 1, 0.0, y, 1)
        torch.cuda.synchronize()
        assert bool((y == float(n)).all()), uplo
    del A, x, y
    torch.cuda.empty_cache()
