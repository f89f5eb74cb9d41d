"""Split-BF16 (tcgen05 tensor core) sgemm / ssymm / ssyrk.

Each FP32 operand is carried as three BF16 terms; results must meet the same
FP32 componentwise bound as the FFMA path (reference grids of
test/level3/{gemm,symm,syrk}/correctness.cpp), and at larger sizes the max
relative error against FP64 must be no worse than the plain FP32 path's."""
import numpy as np
import pytest

from cases import gemm_cases, symm_cases, syr2k_cases, syrk_cases
from common import EPS, check_case, run_gpu


@pytest.fixture
def split_mode(cuda):
    import exoblas_gb300 as eb

    eb.set_precision(eb.PRECISION_SPLIT_BF16)
    yield
    eb.set_precision(eb.PRECISION_NATIVE)


CASES = (
    [c for c in gemm_cases("s", dims=(1, 7, 64, 257), ldds=(0, 5))][::3]
    + [c for c in symm_cases("s", dims=(1, 7, 64, 257))][::2]
    + [c for c in syrk_cases("s", dims=(1, 7, 64, 257))][::2]
    + [c for c in syr2k_cases("s", dims=(1, 7, 64, 257), ldds=(0, 5))][::8]
)


@pytest.mark.gpu
def test_split_bf16_single_tile(split_mode):
    import exoblas_gb300 as eb

    g = np.random.default_rng(1)
    m = n = 128
    k = 64
    A = g.uniform(-1, 1, (m, k)).astype(np.float32)
    B = g.uniform(-1, 1, (k, n)).astype(np.float32)
    C = np.zeros((m, n), np.float32)
    eb.exo_sgemm(101, 111, 111, m, n, k, 1.0, A, k, B, n, 0.0, C, n)
    ref = A.astype(np.float64) @ B.astype(np.float64)
    mag = np.abs(A.astype(np.float64)) @ np.abs(B.astype(np.float64))
    err = np.abs(C - ref) / mag
    assert err.max() <= 4 * k * EPS["s"], err.max()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c.op}-{c.label}")
def test_split_bf16_grid(split_mode, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("stress", [False, True])
def test_split_bf16_error_not_worse_than_ffma(cuda, stress):
    """2048^3 sgemm NN: max relative error vs FP64 (torch double matmul on the
    GPU) of split-BF16 against the FFMA path; inputs uniform[-1,1) or the
    stress set (sign * U[1,2) * 2^e, e uniform in [-16, 16])."""
    import exoblas_gb300 as eb

    torch = cuda
    n = 2048
    gen = torch.Generator(device="cuda").manual_seed(3 if stress else 0)

    def draw():
        if not stress:
            return torch.rand(n, n, device="cuda", generator=gen) * 2 - 1
        sign = torch.where(torch.rand(n, n, device="cuda", generator=gen) < 0.5, -1.0, 1.0)
        mant = 1 + torch.rand(n, n, device="cuda", generator=gen)
        e = torch.randint(-16, 17, (n, n), device="cuda", generator=gen).float()
        return (sign * mant * torch.exp2(e)).float()

    A, B = draw(), draw()
    ref = A.double() @ B.double()
    mag = A.double().abs() @ B.double().abs()
    errs = {}
    for mode in (eb.PRECISION_NATIVE, eb.PRECISION_SPLIT_BF16):
        C = torch.zeros(n, n, device="cuda")
        eb.set_precision(mode)
        try:
            eb.exo_sgemm(101, 111, 111, n, n, n, 1.0, A, n, B, n, 0.0, C, n)
        finally:
            eb.set_precision(eb.PRECISION_NATIVE)
        rel = ((C.double() - ref).abs() / mag).max().item()
        assert rel <= 4 * n * EPS["s"]
        errs[mode] = rel
    print("max componentwise-relative error native / split:", errs)
    assert errs[eb.PRECISION_SPLIT_BF16] <= errs[eb.PRECISION_NATIVE] * 1.05
