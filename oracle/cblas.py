"""ctypes shim over the OpenBLAS bundled with SciPy -- TEST INFRASTRUCTURE ONLY.

The reference checks every exo_* kernel against a system CBLAS
(test/CMakeLists.txt:8-10, README.md:101-105), pinned to one thread
(test/CMakeLists.txt:56,82).  In this container that CBLAS is SciPy's
bundled OpenBLAS (symbols scipy_cblas_*).  It is used to generate the
committed golden fixtures under tests/golden/ and to cross-check the oracle
where it is importable; tests skip it when it is absent.
"""
from __future__ import annotations

import ctypes as C
import glob
import os

_T = {"i": C.c_int, "f": C.c_float, "d": C.c_double, "p": C.c_void_p, "z": C.c_size_t, "v": None}

SIGS = {
    "sasum": ("f", "ipi"), "dasum": ("d", "ipi"),
    "snrm2": ("f", "ipi"), "dnrm2": ("d", "ipi"),
    "isamax": ("z", "ipi"), "idamax": ("z", "ipi"),
    "saxpy": ("v", "ifpipi"), "daxpy": ("v", "idpipi"),
    "sdot": ("f", "ipipi"), "ddot": ("d", "ipipi"),
    "dsdot": ("d", "ipipi"), "sdsdot": ("f", "ifpipi"),
    "scopy": ("v", "ipipi"), "dcopy": ("v", "ipipi"),
    "sswap": ("v", "ipipi"), "dswap": ("v", "ipipi"),
    "sscal": ("v", "ifpi"), "dscal": ("v", "idpi"),
    "srot": ("v", "ipipiff"), "drot": ("v", "ipipidd"),
    "srotm": ("v", "ipipip"), "drotm": ("v", "ipipip"),
    "sgemv": ("v", "iiiifpipifpi"), "dgemv": ("v", "iiiidpipidpi"),
    "sger": ("v", "iiifpipipi"), "dger": ("v", "iiidpipipi"),
    "ssymv": ("v", "iiifpipifpi"), "dsymv": ("v", "iiidpipidpi"),
    "ssyr": ("v", "iiifpipi"), "dsyr": ("v", "iiidpipi"),
    "ssyr2": ("v", "iiifpipipi"), "dsyr2": ("v", "iiidpipipi"),
    "strmv": ("v", "iiiiipipi"), "dtrmv": ("v", "iiiiipipi"),
    "strsv": ("v", "iiiiipipi"), "dtrsv": ("v", "iiiiipipi"),
    "sgemm": ("v", "iiiiiifpipifpi"), "dgemm": ("v", "iiiiiidpipidpi"),
    "ssymm": ("v", "iiiiifpipifpi"), "dsymm": ("v", "iiiiidpipidpi"),
    "ssyrk": ("v", "iiiiifpifpi"), "dsyrk": ("v", "iiiiidpidpi"),
    "ssyr2k": ("v", "iiiiifpipifpi"), "dsyr2k": ("v", "iiiiidpipidpi"),
    "ssbmv": ("v", "iiiifpipifpi"), "dsbmv": ("v", "iiiidpipidpi"),
    "sgbmv": ("v", "iiiiiifpipifpi"), "dgbmv": ("v", "iiiiiidpipidpi"),
    "stbmv": ("v", "iiiiiipipi"), "dtbmv": ("v", "iiiiiipipi"),
    "stbsv": ("v", "iiiiiipipi"), "dtbsv": ("v", "iiiiiipipi"),
    "strmm": ("v", "iiiiiiifpipi"), "dtrmm": ("v", "iiiiiiidpipi"),
}

_lib = None


def find() -> str | None:
    pats = [
        "/usr/local/lib/python3*/dist-packages/scipy.libs/libscipy_openblas*.so",
        "/usr/lib/python3*/dist-packages/scipy.libs/libscipy_openblas*.so",
    ]
    try:
        import scipy

        pats.insert(0, os.path.join(os.path.dirname(scipy.__file__) + ".libs", "libscipy_openblas*.so"))
    except ImportError:
        pass
    for p in pats:
        hits = sorted(glob.glob(p))
        if hits:
            return hits[0]
    return None


def available() -> bool:
    try:
        lib()
        return True
    except OSError:
        return False


def lib():
    global _lib
    if _lib is None:
        path = find()
        if path is None:
            raise OSError("SciPy's bundled OpenBLAS was not found")
        L = C.CDLL(path)
        if not hasattr(L, "scipy_cblas_sgemm"):
            raise OSError("bundled OpenBLAS lacks scipy_cblas_* symbols")
        for name, (res, args) in SIGS.items():
            fn = getattr(L, "scipy_cblas_" + name)
            fn.restype = _T[res]
            fn.argtypes = [_T[a] for a in args]
        if hasattr(L, "scipy_openblas_set_num_threads"):
            L.scipy_openblas_set_num_threads.argtypes = [C.c_int]
            L.scipy_openblas_set_num_threads(1)  # test/CMakeLists.txt:56
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    L = lib()
    if hasattr(L, "scipy_openblas_set_num_threads"):
        L.scipy_openblas_set_num_threads(int(n))


def call(name: str, *args):
    res, codes = SIGS[name]
    conv = [(None if v is None else v.ctypes.data) if c == "p" else v for v, c in zip(args, codes)]
    return getattr(lib(), "scipy_cblas_" + name)(*conv)
