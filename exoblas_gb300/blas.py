"""Python mirror of the exo_<p><op> interface over libexoblas_gb300.so.

Each function has the name, argument order and argument meaning of the
ExoBLAS C++ wrapper it mirrors (test/level*/<op>/exo_<op>_wrapper.h).  Array
arguments may be NumPy arrays (host memory), torch tensors (host or CUDA) or
plain integer addresses; sizes, strides and flags are passed through
unchanged, exactly as a C caller would pass them.

Errors follow the reference: Order != CblasRowMajor raises
UnsupportedParameterException (the reference throws that exception,
test/common/error.h:5-10); other failures raise ExoBlasError.
"""
from __future__ import annotations

import ctypes as C

from . import _native

CblasRowMajor, CblasColMajor = 101, 102
CblasNoTrans, CblasTrans, CblasConjTrans = 111, 112, 113
CblasUpper, CblasLower = 121, 122
CblasNonUnit, CblasUnit = 131, 132
CblasLeft, CblasRight = 141, 142

PRECISION_NATIVE, PRECISION_SPLIT_BF16, PRECISION_OZAKI = 0, 1, 2
CUDA_STREAM_LEGACY = 0x1  # cudaStreamLegacy


class ExoBlasError(RuntimeError):
    def __init__(self, status: int, function: str):
        self.status = status
        msg = _native.lib().exoblas_status_string(status).decode()
        super().__init__(f"{function}: {msg} (status {status})")


class UnsupportedParameterException(ExoBlasError):
    """Order was not CblasRowMajor (the reference throws the same-named C++ exception)."""


_torch_stream = None


def _ptr(a):
    """Address of an array argument (None -> NULL)."""
    global _torch_stream
    if a is None:
        return None
    if isinstance(a, int):
        return a
    mod = type(a).__module__
    if mod.startswith("numpy"):
        if not a.flags["C_CONTIGUOUS"] and a.ndim > 1:
            raise ValueError("numpy operands must be C-contiguous buffers")
        return a.ctypes.data
    if mod.startswith("torch"):
        if a.is_cuda:
            import torch

            # torch's default stream is the legacy default stream (handle 0);
            # the library takes it as cudaStreamLegacy (0x1), NULL meaning the
            # library's own stream
            s = torch.cuda.current_stream(a.device).cuda_stream or CUDA_STREAM_LEGACY
            if s != _torch_stream:
                # run this library's kernels on torch's current stream so they
                # are ordered after the kernels that produced the tensors
                _native.lib().exoblas_set_stream(s)
                _torch_stream = s
        return a.data_ptr()
    if hasattr(a, "__array_interface__"):
        return a.__array_interface__["data"][0]
    raise TypeError(f"unsupported array argument of type {type(a)}")


def _check(name: str):
    st = _native.lib().exoblas_get_status()
    if st == 1:
        raise UnsupportedParameterException(st, name)
    if st != 0:
        raise ExoBlasError(st, name)


def _make(name: str):
    res, args = _native.SIGNATURES[name]

    def fn(*argv):
        if len(argv) != len(args):
            raise TypeError(f"{name} takes {len(args)} arguments ({len(argv)} given)")
        conv = [_ptr(v) if code == "p" else v for v, code in zip(argv, args)]
        out = getattr(_native.lib(), name)(*conv)
        _check(name)
        return out

    fn.__name__ = name
    fn.__qualname__ = name
    fn.__doc__ = f"{name}: see include/exoblas.h for the C declaration and reference citation."
    return fn


_EXO = [n for n in _native.SIGNATURES if n.startswith("exo_")]
for _n in _EXO:
    globals()[_n] = _make(_n)


def set_precision(mode: int) -> None:
    _native.lib().exoblas_set_precision(int(mode))
    _check("exoblas_set_precision")


def get_precision() -> int:
    return _native.lib().exoblas_get_precision()


def set_column_major(enable: bool) -> None:
    """Accept CblasColMajor calls on this thread (rejected by default, as in
    the reference)."""
    _native.lib().exoblas_set_column_major(1 if enable else 0)


def set_blocking(blocking: bool) -> None:
    _native.lib().exoblas_set_blocking(1 if blocking else 0)
    _check("exoblas_set_blocking")


def set_stream(stream) -> None:
    """Use a CUDA stream for this thread's calls: a torch.cuda.Stream (its
    default stream maps to cudaStreamLegacy), a raw cudaStream_t handle, or
    None for the library's own non-blocking stream."""
    global _torch_stream
    if stream is None:
        handle = None
    elif hasattr(stream, "cuda_stream"):
        handle = stream.cuda_stream or CUDA_STREAM_LEGACY
    else:
        handle = int(stream)
    _native.lib().exoblas_set_stream(handle)
    _check("exoblas_set_stream")
    _torch_stream = handle


def synchronize() -> None:
    _native.lib().exoblas_synchronize()
    _check("exoblas_synchronize")


def kernel_launches() -> int:
    return int(_native.lib().exoblas_kernel_launches())


def status() -> int:
    return _native.lib().exoblas_get_status()


def _device_reduce(name):
    def fn(N, X, incX, *rest):
        conv = [N, _ptr(X), incX] + [(_ptr(v) if i % 2 == 0 else v) for i, v in enumerate(rest[:-1])]
        conv.append(_ptr(rest[-1]))
        st = getattr(_native.lib(), name)(*conv)
        if st:
            raise ExoBlasError(st, name)

    fn.__name__ = name
    return fn


exoblas_sasum_device = _device_reduce("exoblas_sasum_device")
exoblas_dasum_device = _device_reduce("exoblas_dasum_device")
exoblas_sdot_device = _device_reduce("exoblas_sdot_device")
exoblas_ddot_device = _device_reduce("exoblas_ddot_device")
exoblas_dsdot_device = _device_reduce("exoblas_dsdot_device")

__all__ = _EXO + [
    "ExoBlasError",
    "UnsupportedParameterException",
    "set_precision",
    "set_column_major",
    "get_precision",
    "set_blocking",
    "set_stream",
    "synchronize",
    "kernel_launches",
    "status",
    "exoblas_sasum_device",
    "exoblas_dasum_device",
    "exoblas_sdot_device",
    "exoblas_ddot_device",
    "exoblas_dsdot_device",
] + [k for k in list(globals()) if k.startswith("Cblas") or k.startswith("PRECISION_")]
