"""Loader for libmma_gb300.so (the CUDA kernels behind every public entry point).

There is no CPU fallback: if the library is missing or cannot be loaded, or no
CUDA device is present, the calls raise instead of computing anything on the host.
"""
import ctypes
import os

_PKG = os.path.dirname(os.path.abspath(__file__))
_LIB = None


class MMAUnavailable(RuntimeError):
    pass


def lib_path():
    return os.path.join(_PKG, "libmma_gb300.so")


def load(build_if_missing=True):
    """Load (building first if needed) the GPU library and return the ctypes handle."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if build_if_missing:
        from .build import build, up_to_date

        if not up_to_date():
            build()
    if not os.path.exists(p):
        raise MMAUnavailable("libmma_gb300.so is not built (run mma_gb300/build.py); there is no CPU fallback")
    _LIB = ctypes.CDLL(p)
    return _LIB
