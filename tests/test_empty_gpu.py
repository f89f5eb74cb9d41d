"""Empty and degenerate sizes (N, M or K of 0 and 1) through every entry
point, compared with the oracle exactly as the reference grids are: the
reference's own tests never go below N = 2, but CBLAS callers do, and the
wrappers' early returns (and gemv's and level 3's beta scaling with nothing
to add) must match."""
import pytest

import cases
from common import check_case, run_gpu


def _level1(ns):
    old = cases.L1_N
    cases.L1_N = list(ns)
    try:
        out = []
        for p in "sd":
            for b in (cases.asum_cases, cases.axpy_cases, cases.dot_cases, cases.copy_cases, cases.swap_cases,
                      cases.scal_cases, cases.rot_cases, cases.rotm_cases):
                out += list(b(p))
        out += list(cases.dsdot_cases()) + list(cases.sdsdot_cases())
        return out
    finally:
        cases.L1_N = old


def _empty_cases():
    out = _level1((0, 1))
    for p in "sd":
        out += list(cases.gemv_cases(p, Ns=(0, 1, 5), Ms=(0, 1, 7)))
        out += list(cases.ger_cases(p, Ms=(0, 1), Ns=(0, 5)))
        out += list(cases.symv_cases(p, Ns=(0, 1)))
        out += list(cases.syr_cases(p, Ns=(0, 1)))
        out += list(cases.syr2_cases(p, Ns=(0, 1)))
        out += list(cases.trmv_cases(p, Ns=(0, 1)))
        out += list(cases.trsv_cases(p, Ns=(0, 1)))
        out += list(cases.gemm_cases(p, dims=(0, 1, 3), ldds=(0,)))
        out += list(cases.symm_cases(p, dims=(0, 1, 3), ldds=(0,)))
        out += list(cases.syrk_cases(p, dims=(0, 1, 3), ldds=(0,)))
        out += list(cases.syr2k_cases(p, dims=(0, 1, 3), ldds=(0,)))
        out += list(cases.tbmv_cases(p, Ns=(1,), Ks=(0,)))  # the band width needs n >= 1
        out += list(cases.tbsv_cases(p, Ns=(1,), Ks=(0,)))  # the band width needs n >= 1
    out += list(cases.trmm_cases(Ms=(0, 1, 4), Ns=(0, 1, 8), alphas=(1.4,), ldds=(0,)))
    return out


EMPTY = _empty_cases()


def test_empty_cases_run_on_the_oracle():
    """The degenerate grid is well formed: the oracle runs every case."""
    from common import run_oracle

    assert len(EMPTY) > 400
    for c in EMPTY:
        run_oracle(c)


@pytest.mark.gpu
@pytest.mark.parametrize("case", EMPTY, ids=lambda c: f"{c.op}-{c.label}")
def test_empty_and_degenerate_sizes(cuda, case):
    r, a = run_gpu(case)
    check_case(case, r, a)


EMPTY_L3 = [c for c in EMPTY if c.op[1:] in ("gemm", "symm", "syrk", "syr2k")]


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2], ids=["split_bf16", "ozaki"])
def test_degenerate_level3_on_precision_paths(cuda, mode):
    """The same degenerate level-3 shapes on the split-BF16 (FP32) and Ozaki
    (FP64) paths: K = 0 takes the native kernels, and 1 x 1 or 3 x 3 outputs
    ride the tensor-core kernels with padded tiles."""
    import exoblas_gb300 as eb

    eb.set_precision(mode)
    try:
        for case in EMPTY_L3:
            r, a = run_gpu(case)
            check_case(case, r, a)
    finally:
        eb.set_precision(0)
