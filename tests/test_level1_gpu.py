"""Level-1 parity on the GPU: exo_<p><op> against the oracle (1% rule),
against FP64 (componentwise bound) and bit-exactly for copy, swap, scal(+-1).
Grids follow test/level1/*/correctness.cpp of the reference."""
import numpy as np
import pytest

from cases import level1_cases
from common import check_case, run_gpu

CASES = list(level1_cases())


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c.op}-{c.label}")
def test_level1_host_pointers(cuda, case):
    r, a = run_gpu(case, device=False)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in CASES if c.args[0] == 1000], ids=lambda c: f"{c.op}-{c.label}")
def test_level1_device_pointers(cuda, case):
    r, a = run_gpu(case, device=True)
    check_case(case, r, a)


@pytest.mark.gpu
def test_reductions_deterministic(cuda):
    import exoblas_gb300 as eb

    g = np.random.default_rng(3)
    x = cuda.from_numpy(g.uniform(-1, 1, 1 << 22).astype(np.float32)).cuda()
    y = cuda.from_numpy(g.uniform(-1, 1, 1 << 22).astype(np.float32)).cuda()
    r = {eb.exo_sdot(1 << 22, x, 1, y, 1) for _ in range(5)}
    d = {eb.exo_dsdot(1 << 22, x, 1, y, 1) for _ in range(5)}
    assert len(r) == 1 and len(d) == 1


@pytest.mark.gpu
def test_misaligned_offsets(cuda):
    """Unit-stride operands that start off a 16-byte boundary (head/tail path)."""
    import exoblas_gb300 as eb
    import oracle

    g = np.random.default_rng(5)
    for off_x, off_y in [(1, 1), (1, 2), (3, 0)]:
        n = 1003
        x = g.uniform(-1, 1, n + 8).astype(np.float32)
        y = g.uniform(-1, 1, n + 8).astype(np.float32)
        dx, dy = cuda.from_numpy(x).cuda(), cuda.from_numpy(y).cuda()
        eb.exo_saxpy(n, 0.5, dx[off_x:], 1, dy[off_y:], 1)
        ref = y.copy()
        oracle.call("saxpy", n, 0.5, x[off_x:], 1, ref[off_y:], 1)
        np.testing.assert_allclose(dy.cpu().numpy(), ref, rtol=1e-6, atol=1e-6)
        got = eb.exo_sdot(n, dx[off_x:], 1, dy[off_y:], 1)
        exp = oracle.call("ddot", n, x[off_x:off_x + n].astype(np.float64), 1, ref[off_y:off_y + n].astype(np.float64), 1)
        assert abs(got - exp) <= 4 * n * np.finfo(np.float32).eps * np.sum(np.abs(x[off_x:off_x + n] * ref[off_y:off_y + n]))


@pytest.mark.gpu
def test_bandwidth_sizes_properties(cuda):
    """Full-size level-1 config (saxpy/sdot/dsdot n=2^26, daxpy/ddot n=2^25):
    results against FP64 / double-double references computed on the GPU in
    torch fp64 (sum order differs, within the componentwise bound)."""
    import exoblas_gb300 as eb

    torch = cuda
    gen = torch.Generator(device="cuda").manual_seed(0)
    n = 1 << 26
    x = torch.rand(n, device="cuda", generator=gen, dtype=torch.float32) * 2 - 1
    y = torch.rand(n, device="cuda", generator=gen, dtype=torch.float32) * 2 - 1
    ref = torch.dot(x.double(), y.double()).item()
    mag = torch.dot(x.double().abs(), y.double().abs()).item()
    got = eb.exo_sdot(n, x, 1, y, 1)
    assert abs(got - ref) <= 4 * n * np.finfo(np.float32).eps * mag
    got = eb.exo_dsdot(n, x, 1, y, 1)
    assert abs(got - ref) <= 4 * n * np.finfo(np.float64).eps * mag
    y2 = y.clone()
    eb.exo_saxpy(n, 0.75, x, 1, y2, 1)
    exp = y.double() + 0.75 * x.double()
    assert torch.all((y2.double() - exp).abs() <= 2 * np.finfo(np.float32).eps * (y.double().abs() + 0.75 * x.double().abs()))
    n = 1 << 25
    xd, yd = x[:n].double(), y[:n].double()
    got = eb.exo_ddot(n, xd, 1, yd, 1)
    assert abs(got - torch.dot(xd, yd).item()) <= 4 * n * np.finfo(np.float64).eps * torch.dot(xd.abs(), yd.abs()).item()


@pytest.mark.gpu
def test_int_max_length_vectors(cuda):
    """N = 2^31 - 1, the largest the int-typed CBLAS signatures carry, on
    device operands (8 GiB each): exact size-independent properties, so
    every element and every index path (32-bit loop indices included) is
    exercised without a CPU oracle of that size."""
    import torch

    import exoblas_gb300 as eb

    n = 2**31 - 1
    x = torch.ones(n, dtype=torch.float32, device="cuda")
    y = torch.full((n,), 2.0, dtype=torch.float32, device="cuda")
    eb.exo_saxpy(n, 3.0, x, 1, y, 1)  # every y becomes 5 exactly
    torch.cuda.synchronize()
    assert bool((y == 5.0).all())
    assert float(y[-1]) == 5.0 and float(y[0]) == 5.0
    # asum of 5s: partial sums stay exact in FP32 up to 2^24, the total rounds once
    r = eb.exo_sasum(n, y, 1)
    assert abs(r - 5.0 * n) <= 5.0 * n * 2**-20
    # i?amax: the single largest element sits at the last index
    y[-1] = 7.0
    assert eb.exo_isamax(n, y, 1) == n - 1
    del x, y
    torch.cuda.empty_cache()
