"""CPU-side checks of the C ABI: the library loads and exports every symbol
include/exoblas.h declares (no GPU calls)."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "exoblas.h").read_text()
    return sorted(set(re.findall(r"EXOBLAS_API\s+[^;(]*?\b((?:exo|exoblas)_\w+)\s*\(", text)))


def test_header_declares_reference_surface():
    syms = declared_symbols()
    ops = ["asum", "axpy", "dot", "copy", "swap", "scal", "rot", "rotm", "gemv", "ger", "symv", "syr", "syr2",
           "trmv", "trsv", "gemm", "symm", "syrk"]
    for p in "sd":
        for op in ops:
            assert f"exo_{p}{op}" in syms, f"exo_{p}{op} not declared"
    assert "exo_dsdot" in syms and "exo_sdsdot" in syms


def test_library_exports_every_declared_symbol():
    import ctypes

    from exoblas_gb300 import _native

    lib = ctypes.CDLL(str(_native.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_binding_table_matches_header():
    from exoblas_gb300 import _native

    assert set(declared_symbols()) == set(_native.SIGNATURES)
