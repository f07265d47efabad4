"""ctypes binding of libsqaod_gb300.so (the C ABI in include/sqaod_gb300.h).

The library is the only compute path: when it cannot be loaded (not built,
or no CUDA driver), importing a solver raises instead of falling back to
anything else.
"""
import ctypes
import os

from . import build as _build

_lib = None


class SqaodError(RuntimeError):
    """Error raised by the native solvers (the reference raises RuntimeError)."""


def lib():
    global _lib
    if _lib is not None:
        return _lib
    path = _build.lib_path()
    if not os.path.exists(path) or not _build._up_to_date(path):
        _build.build()
    L = ctypes.CDLL(path)
    L.sq103_last_error.restype = ctypes.c_char_p
    L.sq103_bf_workspace_bytes.restype = ctypes.c_size_t
    _lib = L
    return L


def call(fn, *args):
    """Calls a handle-layer entry point and raises SqaodError on failure."""
    rc = fn(*args)
    if rc != 0:
        msg = lib().sq103_last_error()
        msg = msg.decode() if msg else "error %d" % rc
        raise SqaodError(msg)
    return rc


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)
