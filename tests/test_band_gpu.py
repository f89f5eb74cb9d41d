"""Banded level 2 on the GPU: gbmv, sbmv, tbmv, tbsv over the grids of
test/level2/{s,d}{gbmv,sbmv,tbmv,tbsv}/correctness.cpp, against the oracle
(the reference's relative rule: 0.1% for gbmv, 1% for the others), FP64
(componentwise bound; double-word for d-precision) and, for the solves, the
residual (its product in double-word for dtbsv)."""
import numpy as np
import pytest

from cases import gbmv_cases, sbmv_cases, tbmv_cases, tbsv_cases
from common import assert_rel1pct, check_case, run_gpu, run_oracle, tbsv_residual_ok

GBMV = [c for p in "sd" for c in gbmv_cases(p, incs=((1, 1), (2, -3)))]
SBMV = [c for p in "sd" for c in sbmv_cases(p)]
TBMV = [c for p in "sd" for c in tbmv_cases(p)]
TBSV = [c for p in "sd" for c in tbsv_cases(p)]


@pytest.mark.gpu
@pytest.mark.parametrize("case", GBMV, ids=lambda c: f"{c.op}-{c.label}")
def test_gbmv(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)
    _, o = run_oracle(case)
    e = o[10].astype(np.float64)
    assert np.all(np.abs(a[10] - e) / np.maximum(1.0, np.abs(e)) < 1e-3), f"{case}: 0.1% rule"


@pytest.mark.gpu
@pytest.mark.parametrize("case", SBMV, ids=lambda c: f"{c.op}-{c.label}")
def test_sbmv(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", TBMV, ids=lambda c: f"{c.op}-{c.label}")
def test_tbmv(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


@pytest.mark.gpu
@pytest.mark.parametrize("case", TBSV, ids=lambda c: f"{c.op}-{c.label}")
def test_tbsv(cuda, case):
    r, a = run_gpu(case)
    _, o = run_oracle(case)
    assert_rel1pct(a[8], o[8], f"{case}")  # the reference's own check
    tbsv_residual_ok(case, a[8])


@pytest.mark.gpu
@pytest.mark.parametrize("case", (GBMV[::3] + SBMV[::40] + TBMV[::40] + TBSV[::40]),
                         ids=lambda c: f"{c.op}-{c.label}")
def test_band_device_pointers(cuda, case):
    r, a = run_gpu(case, device=True)
    if case.op.endswith("tbsv"):
        _, o = run_oracle(case)
        assert_rel1pct(a[8], o[8], f"{case}")
        tbsv_residual_ok(case, a[8])
    else:
        check_case(case, r, a)
