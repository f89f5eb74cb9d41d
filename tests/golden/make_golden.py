"""Generate the golden fixtures under tests/golden/ (run in a container where
SciPy's bundled OpenBLAS is importable).

The reference's correctness tests compare every exo_* kernel against a
system CBLAS at 1% relative error (test/common/correctness_helpers.h:9-16,
test/CMakeLists.txt:8-10) on random inputs, so it ships no golden vectors.
These fixtures freeze that comparison: seeded inputs from subsets of the
reference's parameter grids (tests/cases.py) together with the outputs of
OpenBLAS (scipy_cblas_*, one thread, as test/CMakeLists.txt:56 pins it),
plus the reference's one deterministic fixture (trsv with A = 2.0 and
X[i] = i, test/level2/trsv/correctness.cpp:20-25).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE.parent), str(HERE.parent.parent)]

import cases as C  # noqa: E402
from common import run_cblas  # noqa: E402


def subset(gen, every, limit_elems=1 << 12):
    out = []
    for i, c in enumerate(gen):
        if i % every:
            continue
        if sum(a.size for a in c.args if isinstance(a, np.ndarray)) > limit_elems:
            continue
        out.append(c)
    return out


def families():
    f = {}
    f["level1"] = subset(C.level1_cases(), 2, 1 << 11)
    f["gemv"] = subset((c for p in "sd" for c in C.gemv_cases(p, Ns=(3, 41, 101), Ms=(77, 103))), 3)
    f["ger"] = subset((c for p in "sd" for c in C.ger_cases(p, Ms=(77, 103), Ns=(41, 101))), 3)
    f["symv"] = subset((c for p in "sd" for c in C.symv_cases(p, Ns=(2, 100))), 4)
    f["syr"] = subset((c for p in "sd" for c in C.syr_cases(p, Ns=(2, 100))), 2)
    f["syr2"] = subset((c for p in "sd" for c in C.syr2_cases(p, Ns=(2, 100))), 2)
    f["trmv"] = subset((c for p in "sd" for c in C.trmv_cases(p, Ns=(2, 100))), 3)
    f["trsv"] = subset((c for p in "sd" for c in C.trsv_cases(p, Ns=(2, 100))), 3) + \
        subset((c for p in "sd" for c in C.trsv_cases(p, Ns=(2, 100), fixture=True)), 2)
    f["gemm"] = subset((c for p in "sd" for c in C.gemm_cases(p, dims=(1, 7, 32, 64))), 7)
    f["symm"] = subset((c for p in "sd" for c in C.symm_cases(p, dims=(1, 7, 32, 64))), 5)
    f["syrk"] = subset((c for p in "sd" for c in C.syrk_cases(p, dims=(1, 7, 32, 64))), 5)
    f["syr2k"] = subset((c for p in "sd" for c in C.syr2k_cases(p, dims=(1, 7, 32))), 7)
    f["trmm"] = subset(C.trmm_cases(Ms=(4, 33), Ns=(8, 15)), 3)
    f["gbmv"] = subset((c for p in "sd" for c in C.gbmv_cases(p, sizes=((2, 2, 1, 1), (15, 20, 0, 5), (40, 33, 7, 3)),
                                                            incs=((1, 1), (2, -3)))), 1)
    f["sbmv"] = subset((c for p in "sd" for c in C.sbmv_cases(p, Ns=(2, 100), Ks=(0, 1, 50))), 5)
    f["tbmv"] = subset((c for p in "sd" for c in C.tbmv_cases(p, Ns=(2, 100))), 5)
    f["tbsv"] = subset((c for p in "sd" for c in C.tbsv_cases(p, Ns=(2, 100))), 5)
    f["nrm2"] = subset((c for p in "sd" for c in C.nrm2_cases(p, Ns=(1, 2, 7, 100, 1000))), 1)
    f["iamax"] = subset((c for p in "sd" for c in C.iamax_cases(p, Ns=(1, 2, 7, 100, 1000))), 1)
    return f


def save(name, cases):
    arrays, spec = {}, []
    for i, c in enumerate(cases):
        r, out = run_cblas(c)
        args = []
        for j, a in enumerate(c.args):
            if isinstance(a, np.ndarray):
                key = f"c{i}_a{j}"
                arrays[key] = a
                args.append({"array": key})
            else:
                args.append(a)
        outs = {}
        for j in c.outputs:
            key = f"c{i}_o{j}"
            arrays[key] = out[j]
            outs[str(j)] = key
        spec.append({"op": c.op, "label": c.label, "args": args, "outputs": outs, "scalar": c.scalar,
                     "result": None if r is None else float(r), "nred": c.nred, "exact": c.exact})
    arrays["spec"] = np.frombuffer(json.dumps(spec).encode(), dtype=np.uint8)
    np.savez_compressed(HERE / f"{name}.npz", **arrays)
    return len(cases)


def main():
    total = 0
    for name, cs in families().items():
        n = save(name, cs)
        total += n
        print(f"{name}: {n} cases")
    print("total", total)


if __name__ == "__main__":
    main()
