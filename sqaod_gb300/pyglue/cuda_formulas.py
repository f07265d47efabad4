"""cuda_formulas: the method table of sqaodc/pyglue/formulas.inc:586-605
(CUDA_FORMULAS) on the formula sets of libsqaod_gb300.so.  As in the
reference, the callers (sqaodpy/sqaod/common/formulas_base.py) pass the output
arrays first -- E, or h, J, c -- and the functions write into them."""
import numpy as np

from ..cuda import formulas as _f
from . import _glue, cuda_device


class _FormulaObject:
    def __init__(self, kind):
        self.kind = kind


def _dg(obj):
    if not isinstance(obj, _FormulaObject) or obj.kind != "dg":
        raise RuntimeError("invalid formula object.")


def _bg(obj):
    if not isinstance(obj, _FormulaObject) or obj.kind != "bg":
        raise RuntimeError("invalid formula object.")


def _out(dst, v):
    dst[...] = np.asarray(v).reshape(dst.shape)


def dg_formulas_new():
    return _FormulaObject("dg")


def dg_formulas_delete(obj):
    _dg(obj)


def dg_formulas_assign_device(obj, devobj):
    _dg(obj)
    cuda_device.assign(devobj)


def dense_graph_calculate_E(obj, E, W, x, dtype):
    _dg(obj)
    _out(E, _f.dense_graph_calculate_E(W, x, _glue.check_dtype(dtype)))


def dense_graph_batch_calculate_E(obj, E, W, x, dtype):
    _dg(obj)
    _out(E, _f.dense_graph_batch_calculate_E(W, x, _glue.check_dtype(dtype)))


def dense_graph_calculate_hamiltonian(obj, h, J, c, W, dtype):
    _dg(obj)
    h1, J1, c1 = _f.dense_graph_calculate_hamiltonian(W, _glue.check_dtype(dtype))
    _out(h, h1)
    _out(J, J1)
    c[0] = c1


def dense_graph_calculate_E_from_spin(obj, E, h, J, c, q, dtype):
    _dg(obj)
    _out(E, _f.dense_graph_calculate_E_from_spin(h, J, c, q, _glue.check_dtype(dtype)))


def dense_graph_batch_calculate_E_from_spin(obj, E, h, J, c, q, dtype):
    _dg(obj)
    _out(E, _f.dense_graph_batch_calculate_E_from_spin(h, J, c, q, _glue.check_dtype(dtype)))


def bg_formulas_new():
    return _FormulaObject("bg")


def bg_formulas_delete(obj):
    _bg(obj)


def bg_formulas_assign_device(obj, devobj):
    _bg(obj)
    cuda_device.assign(devobj)


def bipartite_graph_calculate_E(obj, E, b0, b1, W, x0, x1, dtype):
    _bg(obj)
    _out(E, _f.bipartite_graph_calculate_E(b0, b1, W, x0, x1, _glue.check_dtype(dtype)))


def bipartite_graph_batch_calculate_E(obj, E, b0, b1, W, x0, x1, dtype):
    _bg(obj)
    _out(E, _f.bipartite_graph_batch_calculate_E(b0, b1, W, x0, x1, _glue.check_dtype(dtype)))


def bipartite_graph_batch_calculate_E_2d(obj, E, b0, b1, W, x0, x1, dtype):
    _bg(obj)
    _out(E, _f.bipartite_graph_batch_calculate_E_2d(b0, b1, W, x0, x1, _glue.check_dtype(dtype)))


def bipartite_graph_calculate_hamiltonian(obj, h0, h1, J, c, b0, b1, W, dtype):
    _bg(obj)
    a, b, J1, c1 = _f.bipartite_graph_calculate_hamiltonian(b0, b1, W, _glue.check_dtype(dtype))
    _out(h0, a)
    _out(h1, b)
    _out(J, J1)
    c[0] = c1


def bipartite_graph_calculate_E_from_spin(obj, E, h0, h1, J, c, q0, q1, dtype):
    _bg(obj)
    _out(E, _f.bipartite_graph_calculate_E_from_spin(h0, h1, J, c, q0, q1, _glue.check_dtype(dtype)))


def bipartite_graph_batch_calculate_E_from_spin(obj, E, h0, h1, J, c, q0, q1, dtype):
    _bg(obj)
    _out(E, _f.bipartite_graph_batch_calculate_E_from_spin(h0, h1, J, c, q0, q1, _glue.check_dtype(dtype)))
