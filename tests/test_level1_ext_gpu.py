"""nrm2 and i?amax on the GPU (no reference counterpart, README.md:15):
nrm2 within the componentwise FP64 bound (including FP64 magnitudes whose
squares overflow or underflow), i?amax bit-exact against the oracle's
sequential first-index rule."""
import numpy as np
import pytest

from cases import iamax_cases, nrm2_cases
from common import check_case, run_gpu, run_oracle

NRM2 = [c for p in "sd" for c in nrm2_cases(p)]
IAMAX = [c for p in "sd" for c in iamax_cases(p)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", NRM2, ids=lambda c: f"{c.op}-{c.label}")
def test_nrm2(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", IAMAX, ids=lambda c: f"{c.op}-{c.label}")
def test_iamax(cuda, case):
    r, _ = run_gpu(case)
    o, _ = run_oracle(case)
    assert int(r) == int(o), f"{case}: {r} != {o}"


@pytest.mark.gpu
def test_nrm2_iamax_nonfinite(cuda):
    import exoblas_gb300 as eb

    x = np.array([1.0, np.inf, 2.0, 3.0])
    assert eb.exo_dnrm2(4, x, 1) == np.inf
    x = np.array([1.0, np.nan, 2.0])
    assert np.isnan(eb.exo_dnrm2(3, x, 1))
    x = np.array([1.0, np.nan, 3.0, -3.0])
    assert eb.exo_idamax(4, x, 1) == 2  # NaN never wins, first of equal magnitudes
    x = np.array([np.nan, 5.0, 7.0])
    assert eb.exo_idamax(3, x, 1) == 0  # the sequential loop starts from |x[0]|
