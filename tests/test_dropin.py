"""The reference's own correctness programs, compiled unchanged against this
library: the drop-in check for a C/C++ caller.

Each test/level{1,2,3}/<op>/correctness.cpp of exo-lang/ExoBLAS includes
its wrapper header (exo_<op>_wrapper.h, or exo_<op>.h for the banded ops,
strmm and sdsdot), the reference's cblas.h and test helpers, and calls
exo_<p><op> beside cblas_<p><op> (test/common/misc.h:138-172,
generate_wrapper).  Here every wrapper header is replaced by a one-line
header that includes include/exoblas.h, the cblas_* functions forward to the
OpenBLAS bundled with SciPy (its symbols are scipy_cblas_*), and the program
is linked against libexoblas_gb300.so.  The .cpp sources and the test/common
helpers are read from the reference tree where it exists; nothing of it is
copied into this repository.

On a machine without a GPU the test compiles and links every program (the
ABI check: same names, argument types and flag enums).  Running them needs
a GB300: build_programs() is the same build, used for that run.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
REF_TESTS = Path(os.environ.get("EXOBLAS_REFERENCE_TESTS", "/root/reference/test"))

# cblas_* routines the programs call, as (return type, name, parameter list);
# each forwards to scipy_cblas_<name>.
_E = "const enum CBLAS_ORDER"
_T = "const enum CBLAS_TRANSPOSE"
_U = "const enum CBLAS_UPLO"
_D = "const enum CBLAS_DIAG"
_S = "const enum CBLAS_SIDE"
SIGS = []
for p, t in (("s", "float"), ("d", "double")):
    SIGS += [
        (t, f"{p}asum", f"const int N, const {t} *X, const int incX"),
        ("void", f"{p}axpy", f"const int N, const {t} alpha, const {t} *X, const int incX, {t} *Y, const int incY"),
        ("void", f"{p}copy", f"const int N, const {t} *X, const int incX, {t} *Y, const int incY"),
        (t, f"{p}dot", f"const int N, const {t} *X, const int incX, const {t} *Y, const int incY"),
        ("void", f"{p}rot", f"const int N, {t} *X, const int incX, {t} *Y, const int incY, const {t} c, const {t} s"),
        ("void", f"{p}rotm", f"const int N, {t} *X, const int incX, {t} *Y, const int incY, const {t} *P"),
        ("void", f"{p}scal", f"const int N, const {t} alpha, {t} *X, const int incX"),
        ("void", f"{p}swap", f"const int N, {t} *X, const int incX, {t} *Y, const int incY"),
        ("void", f"{p}gemv", f"{_E} order, {_T} TransA, const int M, const int N, const {t} alpha, const {t} *A, "
                             f"const int lda, const {t} *X, const int incX, const {t} beta, {t} *Y, const int incY"),
        ("void", f"{p}gbmv", f"{_E} order, {_T} TransA, const int M, const int N, const int KL, const int KU, "
                             f"const {t} alpha, const {t} *A, const int lda, const {t} *X, const int incX, "
                             f"const {t} beta, {t} *Y, const int incY"),
        ("void", f"{p}ger", f"{_E} order, const int M, const int N, const {t} alpha, const {t} *X, const int incX, "
                            f"const {t} *Y, const int incY, {t} *A, const int lda"),
        ("void", f"{p}symv", f"{_E} order, {_U} Uplo, const int N, const {t} alpha, const {t} *A, const int lda, "
                             f"const {t} *X, const int incX, const {t} beta, {t} *Y, const int incY"),
        ("void", f"{p}sbmv", f"{_E} order, {_U} Uplo, const int N, const int K, const {t} alpha, const {t} *A, "
                             f"const int lda, const {t} *X, const int incX, const {t} beta, {t} *Y, const int incY"),
        ("void", f"{p}syr", f"{_E} order, {_U} Uplo, const int N, const {t} alpha, const {t} *X, const int incX, "
                            f"{t} *A, const int lda"),
        ("void", f"{p}syr2", f"{_E} order, {_U} Uplo, const int N, const {t} alpha, const {t} *X, const int incX, "
                             f"const {t} *Y, const int incY, {t} *A, const int lda"),
        ("void", f"{p}trmv", f"{_E} order, {_U} Uplo, {_T} TransA, {_D} Diag, const int N, const {t} *A, "
                             f"const int lda, {t} *X, const int incX"),
        ("void", f"{p}trsv", f"{_E} order, {_U} Uplo, {_T} TransA, {_D} Diag, const int N, const {t} *A, "
                             f"const int lda, {t} *X, const int incX"),
        ("void", f"{p}tbmv", f"{_E} order, {_U} Uplo, {_T} TransA, {_D} Diag, const int N, const int K, "
                             f"const {t} *A, const int lda, {t} *X, const int incX"),
        ("void", f"{p}tbsv", f"{_E} order, {_U} Uplo, {_T} TransA, {_D} Diag, const int N, const int K, "
                             f"const {t} *A, const int lda, {t} *X, const int incX"),
        ("void", f"{p}gemm", f"{_E} Order, {_T} TransA, {_T} TransB, const int M, const int N, const int K, "
                             f"const {t} alpha, const {t} *A, const int lda, const {t} *B, const int ldb, "
                             f"const {t} beta, {t} *C, const int ldc"),
        ("void", f"{p}symm", f"{_E} Order, {_S} Side, {_U} Uplo, const int M, const int N, const {t} alpha, "
                             f"const {t} *A, const int lda, const {t} *B, const int ldb, const {t} beta, {t} *C, "
                             f"const int ldc"),
        ("void", f"{p}syrk", f"{_E} Order, {_U} Uplo, {_T} Trans, const int N, const int K, const {t} alpha, "
                             f"const {t} *A, const int lda, const {t} beta, {t} *C, const int ldc"),
        ("void", f"{p}syr2k", f"{_E} Order, {_U} Uplo, {_T} Trans, const int N, const int K, const {t} alpha, "
                              f"const {t} *A, const int lda, const {t} *B, const int ldb, const {t} beta, {t} *C, "
                              f"const int ldc"),
        ("void", f"{p}trmm", f"{_E} Order, {_S} Side, {_U} Uplo, {_T} TransA, {_D} Diag, const int M, const int N, "
                             f"const {t} alpha, const {t} *A, const int lda, {t} *B, const int ldb"),
    ]
SIGS += [
    ("double", "dsdot", "const int N, const float *X, const int incX, const float *Y, const int incY"),
    ("float", "sdsdot", "const int N, const float alpha, const float *X, const int incX, const float *Y, "
                        "const int incY"),
]


def _arg_names(params):
    return ", ".join(p.replace("*", " ").split()[-1] for p in params.split(","))


def forwarders_source() -> str:
    """C source: cblas_<name>(...) forwards to scipy_cblas_<name>(...)."""
    lines = ["/* cblas_* -> scipy_cblas_* forwarders (generated by tests/test_dropin.py) */",
             "#include <cblas.h>"]
    for ret, name, params in SIGS:
        call = f"scipy_cblas_{name}({_arg_names(params)})"
        lines.append(f"{ret} scipy_cblas_{name}({params});")
        body = f"return {call};" if ret != "void" else f"{call};"
        lines.append(f"{ret} cblas_{name}({params}) {{ {body} }}")
    return "\n".join(lines) + "\n"


def programs(ref_tests: Path = REF_TESTS):
    """(name, correctness.cpp, wrapper header names it includes)."""
    out = []
    for cpp in sorted(ref_tests.glob("level*/*/correctness.cpp")):
        heads = [l.split('"')[1] for l in cpp.read_text().splitlines()
                 if l.startswith('#include "exo_')]
        out.append((cpp.parent.name, cpp, heads))
    return out


def build_programs(out: Path, ref_tests: Path = REF_TESTS, jobs: int = 8):
    """Compile every reference correctness program against include/exoblas.h
    and link it with libexoblas_gb300.so and the OpenBLAS forwarders.
    Returns {name: executable path}; raises on the first compile error."""
    from concurrent.futures import ThreadPoolExecutor

    from exoblas_gb300 import build as libbuild
    from oracle import cblas

    lib = libbuild.build()
    found = cblas.find()
    if found is None:
        raise RuntimeError("SciPy's bundled OpenBLAS was not found")
    blas = Path(found)
    shim = out / "shim"
    shim.mkdir(parents=True, exist_ok=True)
    progs = programs(ref_tests)
    for _, _, heads in progs:
        for h in heads:
            (shim / h).write_text('#pragma once\n#include "exoblas.h"\n')
    common = ref_tests / "common"
    fwd_c = out / "cblas_forward.c"
    fwd_c.write_text(forwarders_source())
    fwd_o = out / "cblas_forward.o"
    subprocess.run(["gcc", "-O1", "-c", "-fPIC", "-I", str(common), str(fwd_c), "-o", str(fwd_o)], check=True,
                   capture_output=True, text=True)

    def one(item):
        # The source is read from stdin with the shim directory as the
        # working directory: a quoted include then finds the shim's wrapper
        # header before the reference's own (which sits beside the .cpp and
        # needs the Exo-generated headers).
        name, cpp, _ = item
        exe = out / f"{name}_correctness"
        cmd = ["g++", "-std=c++17", "-O1", "-w", "-I", str(shim), "-I", str(ROOT / "include"), "-I", str(common),
               "-x", "c++", "-", "-x", "none", str(fwd_o), "-o", str(exe), str(lib), str(blas),
               f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{blas.parent}"]
        r = subprocess.run(cmd, input=cpp.read_text(), cwd=shim, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{name}: {' '.join(cmd)}\n{r.stderr[-3000:]}")
        return name, exe

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        return dict(ex.map(one, progs))


@pytest.mark.skipif(not (REF_TESTS / "common" / "cblas.h").exists(), reason="reference test tree not present")
def test_reference_correctness_programs_compile_and_link(tmp_path):
    """All 30 reference correctness programs build unchanged against
    include/exoblas.h and link against libexoblas_gb300.so: every exo_*
    name, argument type and flag enum they use is what this library
    exports."""
    pytest.importorskip("scipy")
    exes = build_programs(tmp_path)
    assert len(exes) == len(programs()) == 30
    for exe in exes.values():
        assert exe.exists()
