"""ctypes loader for libexoblas_gb300.so and the table of its C signatures.

The library is built in-tree by exoblas_gb300.build (or __graft_entry__.build)
and loaded from this package directory.  There is no CPU fallback: importing
a function whose library is missing raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libexoblas_gb300.so"

# C type codes used in the signature table
_T = {
    "z": C.c_size_t,
    "i": C.c_int,
    "f": C.c_float,
    "d": C.c_double,
    "p": C.c_void_p,
    "v": None,
    "s": C.c_char_p,
    "u": C.c_ulonglong,
}

L1 = {
    # name: (restype, argtypes)  -- pointers are 'p'
    "exo_sasum": ("f", "ipi"),
    "exo_dasum": ("d", "ipi"),
    "exo_snrm2": ("f", "ipi"),
    "exo_dnrm2": ("d", "ipi"),
    "exo_isamax": ("z", "ipi"),
    "exo_idamax": ("z", "ipi"),
    "exo_saxpy": ("v", "ifpipi"),
    "exo_daxpy": ("v", "idpipi"),
    "exo_sdot": ("f", "ipipi"),
    "exo_ddot": ("d", "ipipi"),
    "exo_dsdot": ("d", "ipipi"),
    "exo_sdsdot": ("f", "ifpipi"),
    "exo_scopy": ("v", "ipipi"),
    "exo_dcopy": ("v", "ipipi"),
    "exo_sswap": ("v", "ipipi"),
    "exo_dswap": ("v", "ipipi"),
    "exo_sscal": ("v", "ifpi"),
    "exo_dscal": ("v", "idpi"),
    "exo_srot": ("v", "ipipiff"),
    "exo_drot": ("v", "ipipidd"),
    "exo_srotm": ("v", "ipipip"),
    "exo_drotm": ("v", "ipipip"),
}
L2 = {
    "exo_sgemv": ("v", "iiiifpipifpi"),
    "exo_dgemv": ("v", "iiiidpipidpi"),
    "exo_sger": ("v", "iiifpipipi"),
    "exo_dger": ("v", "iiidpipipi"),
    "exo_ssymv": ("v", "iiifpipifpi"),
    "exo_dsymv": ("v", "iiidpipidpi"),
    "exo_ssyr": ("v", "iiifpipi"),
    "exo_dsyr": ("v", "iiidpipi"),
    "exo_ssyr2": ("v", "iiifpipipi"),
    "exo_dsyr2": ("v", "iiidpipipi"),
    "exo_strmv": ("v", "iiiiipipi"),
    "exo_dtrmv": ("v", "iiiiipipi"),
    "exo_strsv": ("v", "iiiiipipi"),
    "exo_dtrsv": ("v", "iiiiipipi"),
}
L3 = {
    "exo_sgemm": ("v", "iiiiiifpipifpi"),
    "exo_dgemm": ("v", "iiiiiidpipidpi"),
    "exo_ssymm": ("v", "iiiiifpipifpi"),
    "exo_dsymm": ("v", "iiiiidpipidpi"),
    "exo_ssyrk": ("v", "iiiiifpifpi"),
    "exo_dsyrk": ("v", "iiiiidpidpi"),
    "exo_sgbmv": ("v", "iiiifpipifpi"),
    "exo_dgbmv": ("v", "iiiidpipidpi"),
    "exo_ssbmv": ("v", "iiiifpipifpi"),
    "exo_dsbmv": ("v", "iiiidpipidpi"),
    "exo_stbmv": ("v", "iiiiiipipi"),
    "exo_dtbmv": ("v", "iiiiiipipi"),
    "exo_stbsv": ("v", "iiiiiipipi"),
    "exo_dtbsv": ("v", "iiiiiipipi"),
    "exo_ssyr2k": ("v", "iiiiifpipifpi"),
    "exo_dsyr2k": ("v", "iiiiidpipidpi"),
    "exo_strmm": ("v", "iiiiiiifpipi"),
}
EXTRA = {
    "exoblas_get_status": ("i", ""),
    "exoblas_status_string": ("s", "i"),
    "exoblas_set_error_handler": ("v", "p"),
    "exoblas_set_stream": ("i", "p"),
    "exoblas_get_stream": ("p", ""),
    "exoblas_set_blocking": ("i", "i"),
    "exoblas_synchronize": ("i", ""),
    "exoblas_selftest_wait_timeout": ("i", "d"),
    "exoblas_set_precision": ("i", "i"),
    "exoblas_get_precision": ("i", ""),
    "exoblas_kernel_launches": ("u", ""),
    "exoblas_staged_bytes": ("v", "pp"),
    "exoblas_sasum_device": ("i", "ipip"),
    "exoblas_dasum_device": ("i", "ipip"),
    "exoblas_sdot_device": ("i", "ipipip"),
    "exoblas_ddot_device": ("i", "ipipip"),
    "exoblas_dsdot_device": ("i", "ipipip"),
    "exoblas_snrm2_device": ("i", "ipip"),
    "exoblas_dnrm2_device": ("i", "ipip"),
    "exoblas_isamax_device": ("i", "ipip"),
    "exoblas_idamax_device": ("i", "ipip"),
    "exoblas_sgemv_noalloc": ("i", "iiiifpipifpip"),
    "exoblas_batch_plan_create": ("i", "pip"),
    "exoblas_batch_plan_run": ("i", "p"),
    "exoblas_batch_plan_graph_launch": ("i", "p"),
    "exoblas_batch_plan_info": ("i", "pppp"),
    "exoblas_batch_plan_destroy": ("i", "p"),
    "exoblas_batch_tune": ("i", ""),
    "exoblas_batch_tile_config": ("i", "iii"),
    "exoblas_batch_set_tensor_cores": ("i", "i"),
    "exoblas_batch_plan_tensor_core_calls": ("i", "pp"),
    "exoblas_set_column_major": ("i", "i"),
    "exoblas_get_column_major": ("i", ""),
    "exoblas_server_create": ("i", "izzzp"),
    "exoblas_server_submit": ("i", "ppd"),
    "exoblas_server_now": ("d", ""),
    "exoblas_server_replay": ("i", "pppzp"),
    "exoblas_server_drain": ("i", "p"),
    "exoblas_server_stats": ("i", "pp"),
    "exoblas_server_batch_stats": ("i", "pp"),
    "exoblas_server_destroy": ("i", "p"),
    "exoblas_reserve_scratch": ("i", "z"),
}

SIGNATURES = {**L1, **L2, **L3, **EXTRA}

_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                "(there is no CPU fallback)"
            )
        mode = getattr(os, "RTLD_GLOBAL", 0)
        lib_ = C.CDLL(str(LIB_PATH), mode=mode)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib_, name, None)
            if fn is None:
                continue
            fn.restype = _T[res]
            fn.argtypes = [_T[a] for a in args]
        _lib = lib_
    return _lib


def exported_symbols() -> list[str]:
    """Names from the signature table that the loaded library exports."""
    L = lib()
    return [n for n in SIGNATURES if hasattr(L, n)]
