"""CPU oracle for exoblas_gb300 -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs may import this package, and only as the checker or the timed CPU
baseline: the GPU library never calls it.

Contents
- liboracle.so (built from exo_oracle.cpp): a C++ restatement of every
  in-scope ExoBLAS @proc algorithm and its CBLAS-order wrapper, plus
  double-double reference kernels and threaded drivers for baseline timing.
- cblas: a ctypes shim over the OpenBLAS bundled with SciPy (the reference's
  own comparison library family, test/CMakeLists.txt:8-10), used to pin the
  restatement where it is importable.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "exo_oracle.cpp"
LIB = HERE / "liboracle.so"

# -O3 mirrors the reference presets' optimisation level (CMakePresets.json:
# 41-42, 57-58).  -ffast-math and -march=native are left out: the oracle must
# keep IEEE semantics (NaN propagation through beta = 0) and build the same
# on x86-64 and aarch64 hosts.
CXXFLAGS = ["-O3", "-std=c++17", "-shared", "-fPIC", "-pthread", "-fno-fast-math"]


def _foreign(path: Path) -> bool:
    """True when `path` is not an ELF object for this host's architecture."""
    import platform

    head = path.read_bytes()[:20]
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(platform.machine())
    return head[:4] != b"\x7fELF" or (want is not None and int.from_bytes(head[18:20], "little") != want)


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or _foreign(LIB) or LIB.stat().st_mtime < SRC.stat().st_mtime:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = ["g++", *CXXFLAGS, str(SRC), "-o", str(tmp)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
        tmp.replace(LIB)
    return LIB


_T = {"i": C.c_int, "l": C.c_long, "f": C.c_float, "d": C.c_double, "p": C.c_void_p, "v": None}

SIGS = {
    "oracle_last_status": ("i", ""),
    "oracle_sasum": ("f", "ipi"),
    "oracle_dasum": ("d", "ipi"),
    "oracle_saxpy": ("v", "ifpipi"),
    "oracle_daxpy": ("v", "idpipi"),
    "oracle_sdot": ("f", "ipipi"),
    "oracle_ddot": ("d", "ipipi"),
    "oracle_dsdot": ("d", "ipipi"),
    "oracle_sdsdot": ("f", "ifpipi"),
    "oracle_scopy": ("v", "ipipi"),
    "oracle_dcopy": ("v", "ipipi"),
    "oracle_sswap": ("v", "ipipi"),
    "oracle_dswap": ("v", "ipipi"),
    "oracle_sscal": ("v", "ifpi"),
    "oracle_dscal": ("v", "idpi"),
    "oracle_srot": ("v", "ipipiff"),
    "oracle_drot": ("v", "ipipidd"),
    "oracle_srotm": ("v", "ipipip"),
    "oracle_drotm": ("v", "ipipip"),
    "oracle_sgemv": ("v", "iiiifpipifpi"),
    "oracle_dgemv": ("v", "iiiidpipidpi"),
    "oracle_sger": ("v", "iiifpipipi"),
    "oracle_dger": ("v", "iiidpipipi"),
    "oracle_ssymv": ("v", "iiifpipifpi"),
    "oracle_dsymv": ("v", "iiidpipidpi"),
    "oracle_ssyr": ("v", "iiifpipi"),
    "oracle_dsyr": ("v", "iiidpipi"),
    "oracle_ssyr2": ("v", "iiifpipipi"),
    "oracle_dsyr2": ("v", "iiidpipipi"),
    "oracle_strmv": ("v", "iiiiipipi"),
    "oracle_dtrmv": ("v", "iiiiipipi"),
    "oracle_strsv": ("v", "iiiiipipi"),
    "oracle_dtrsv": ("v", "iiiiipipi"),
    "oracle_sgemm": ("v", "iiiiiifpipifpi"),
    "oracle_dgemm": ("v", "iiiiiidpipidpi"),
    "oracle_ssymm": ("v", "iiiiifpipifpi"),
    "oracle_dsymm": ("v", "iiiiidpipidpi"),
    "oracle_ssyrk": ("v", "iiiiifpifpi"),
    "oracle_dsyrk": ("v", "iiiiidpidpi"),
    "oracle_snrm2": ("f", "ipi"),
    "oracle_dnrm2": ("d", "ipi"),
    "oracle_isamax": ("l", "ipi"),
    "oracle_idamax": ("l", "ipi"),
    "oracle_sgbmv": ("v", "iiiifpipifpi"),
    "oracle_dgbmv": ("v", "iiiidpipidpi"),
    "oracle_ssbmv": ("v", "iiiifpipifpi"),
    "oracle_dsbmv": ("v", "iiiidpipidpi"),
    "oracle_stbmv": ("v", "iiiiiipipi"),
    "oracle_dtbmv": ("v", "iiiiiipipi"),
    "oracle_stbsv": ("v", "iiiiiipipi"),
    "oracle_dtbsv": ("v", "iiiiiipipi"),
    "oracle_ssyr2k": ("v", "iiiiifpipifpi"),
    "oracle_dsyr2k": ("v", "iiiiidpipidpi"),
    "oracle_strmm": ("v", "iiiiiiifpipi"),
    "oracle_dtrmm": ("v", "iiiiiiidpipi"),
    "oracle_dd_dot": ("d", "lplpl"),
    "oracle_dd_gemv": ("v", "illdplpdpp"),
    "oracle_dd_trsv": ("v", "iiilplpp"),
    "oracle_dd_gemm_entries": ("v", "iildplpldplpplp"),
    "oracle_par_saxpy": ("v", "iifpp"),
    "oracle_par_daxpy": ("v", "iidpp"),
    "oracle_par_sdot": ("f", "iipp"),
    "oracle_par_ddot": ("d", "iipp"),
    "oracle_par_dsdot": ("d", "iipp"),
    "oracle_par_sgemv": ("v", "iiiifpipfp"),
    "oracle_par_dtrsv_lnn": ("v", "iipip"),
    "oracle_par_sgemm": ("v", "iiiiiifpipifpi"),
}

# Double-word (about 104-bit) instantiations of the restatements: same
# arguments as the d-variant, every array a {hi, lo} pair array.
DW_OPS = (
    "dasum daxpy ddot dscal drot drotm dgemv dger dsymv dsyr dsyr2 dtrmv dtrsv dgemm dsymm dsyrk "
    "dgbmv dsbmv dtbmv dtbsv dsyr2k dtrmm dnrm2"
).split()
for _op in DW_OPS:
    SIGS["oracle_dw_" + _op] = SIGS["oracle_" + _op]

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        for name, (res, args) in SIGS.items():
            fn = getattr(L, name)
            fn.restype = _T[res]
            fn.argtypes = [_T[a] for a in args]
        _lib = L
    return _lib


def _addr(a):
    if a is None:
        return None
    if isinstance(a, int):
        return a
    return a.ctypes.data


def call(name: str, *args):
    """Call oracle_<name> with NumPy arrays converted to addresses."""
    res, codes = SIGS["oracle_" + name]
    conv = [_addr(v) if c == "p" else v for v, c in zip(args, codes)]
    return getattr(lib(), "oracle_" + name)(*conv)


def last_status() -> int:
    return lib().oracle_last_status()


def call_dw(name: str, *args):
    """Run the double-word instantiation oracle_dw_<name> (name a d-op such as
    "dgemv") on float64 arguments.  Returns (result, args) like a plain call,
    with every array argument replaced by a float64 copy holding the
    double-word result rounded to double; the caller's arrays are untouched."""
    import numpy as np

    res, codes = SIGS["oracle_dw_" + name]
    pairs, conv = [], []
    for v, c in zip(args, codes):
        if c == "p" and v is not None and not isinstance(v, int):
            a = np.asarray(v, np.float64)
            w = np.zeros(a.shape + (2,), np.float64)
            w[..., 0] = a
            pairs.append(w)
            conv.append(w.ctypes.data)
        else:
            pairs.append(None)
            conv.append(v)
    r = getattr(lib(), "oracle_dw_" + name)(*conv)
    out = []
    for v, w in zip(args, pairs):
        if w is None:
            out.append(v)
        else:
            hi, lo = w[..., 0], w[..., 1]
            with np.errstate(invalid="ignore", over="ignore"):
                out.append(np.where(np.isfinite(hi), hi + lo, hi))
    return r, out
