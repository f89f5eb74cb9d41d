"""exoblas_gb300: the ExoBLAS dense BLAS hot path as hand-written sm_103a CUDA.

The product is the C-ABI shared library libexoblas_gb300.so (declared in
include/exoblas.h).  This package builds it (exoblas_gb300.build) and binds
it through ctypes (exoblas_gb300.blas); the batching and serving layers sit
on top of the same library.
"""
from .blas import *  # noqa: F401,F403
from .blas import __all__ as _blas_all

__all__ = list(_blas_all)
