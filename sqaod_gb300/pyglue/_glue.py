"""Helpers shared by the extension-module stand-ins (argument checks of
sqaodc/pyglue/pyglue.h)."""
import numpy as np


def check_dtype(dtype):
    """ASSERT_DTYPE of sqaodc/pyglue/pyglue.h:252-254."""
    try:
        d = np.dtype(dtype)
    except TypeError:
        d = None
    if d not in (np.dtype(np.float32), np.dtype(np.float64)):
        raise RuntimeError("dtype is not float64 nor float32.")
    return d.type


def check_handle(obj, cls):
    if not isinstance(obj, cls):
        raise RuntimeError("invalid solver object.")
    return obj


def to_E(E, dtype):
    return np.asarray(E, dtype=dtype)
