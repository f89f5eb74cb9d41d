"""GPU results against the committed CBLAS golden fixtures (the reference's
own comparison, frozen), with the same checks the oracle is pinned by."""
import pytest

import golden_io
from common import run_gpu
from test_oracle import FIXTURES, check_against, fixture


@pytest.mark.gpu
@pytest.mark.parametrize("name,i", FIXTURES, ids=lambda v: str(v))
def test_gpu_matches_cblas_golden(cuda, name, i):
    case, exp_r, exp_out = fixture(name, i)
    r, a = run_gpu(case)
    check_against(case, r, a, exp_r, exp_out, "gpu")
