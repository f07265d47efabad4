"""sqaod.cuda.formulas on libsqaod_gb300.so.

QUBO and Ising energies and the QUBO -> Ising conversion for dense and
bipartite graphs: the functions, arguments and checks of
sqaodpy/sqaod/cuda/formulas.py over sqaodpy/sqaod/common/formulas_base.py.
Each call goes through one sq103_{dg,bg}_formulas_* entry point of the C ABI,
which uploads the arguments, runs the device kernels and copies the result
back.  Energies are summed in FP64 on the device and returned in `dtype`.

dtype numpy.float32 runs the fp32-input kernels the solvers use (FP64 sums),
numpy.float64 plain FP64 kernels (the reference's <double> instantiation);
other dtypes raise.

Differences from the reference, all deliberate:
  * bits must be 0 / 1 and spins -1 / +1 (the device kernels check);
  * bipartite_graph_batch_calculate_E_2d works for any two batch sizes and
    returns E[i1][i0]; the reference's version always raises (its body reads
    undefined names, sqaodpy/sqaod/common/formulas_base.py:118).
"""
import ctypes

import numpy as np

from .. import common
from .._lib import call, lib, ptr

_c_int = ctypes.c_int


class _FormulaSet:
    """One native formula object (dg_formulas_new / bg_formulas_new)."""

    def __init__(self, prefix):
        self._L = lib()
        self._prefix = prefix
        h = ctypes.c_void_p()
        call(getattr(self._L, '%s_new' % prefix), ctypes.byref(h))
        self._h = h

    def __call__(self, name, *args):
        return call(getattr(self._L, '%s_%s' % (self._prefix, name)), self._h, *args)

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                getattr(self._L, '%s_delete' % self._prefix)(h)
            except Exception:
                pass
            self._h = None


_objs = {}


def _check_dtype(dtype):
    d = np.dtype(np.float32 if dtype is None else dtype)
    if d not in (np.float32, np.float64):
        raise RuntimeError("dtype %s is not provided: the formulas compute in float32 or float64." % d)
    return d.type


def _real(dtype):
    return ctypes.c_double if dtype is np.float64 else ctypes.c_float


def _dg(dtype):
    return _obj('sq103_dg_formulas64' if dtype is np.float64 else 'sq103_dg_formulas')


def _bg(dtype):
    return _obj('sq103_bg_formulas64' if dtype is np.float64 else 'sq103_bg_formulas')


def _obj(prefix):
    o = _objs.get(prefix)
    if o is None:
        o = _objs[prefix] = _FormulaSet(prefix)
    return o


def unload():
    """Releases the native formula objects (the reference's unload())."""
    _objs.clear()


# ------------------------------------------------------------ argument checks
# (sqaodpy/sqaod/common/checkers.py)

def _bits(*arrays):
    for a in arrays:
        if a.dtype != np.int8:
            raise RuntimeError("bits are not given as np.int8")


def _vector(name, v):
    if not (isinstance(v, np.ndarray) and v.ndim == 1):
        raise RuntimeError("%s is not a vector. %s" % (name, type(v)))


def _scalar(name, c):
    if not common.is_scalar(c):
        raise RuntimeError("%s is not a scalar. %s" % (name, type(c)))


def _square(name, W):
    if len(W.shape) != 2 or W.shape[0] != W.shape[1]:
        raise RuntimeError("wrong shape dim=(%s) = %s" % (name, W.shape))


def _dims(caption, *arrays):
    raise RuntimeError("dimension mismatch for %s. %s" % (caption, ", ".join(str(a.shape) for a in arrays)))


def _dense_rows(W, x, caption):
    """x as a C-contiguous (m, N) int8 matrix; 1-D x is one row."""
    _bits(x)
    if x.shape[-1] != W.shape[0]:
        _dims(caption, W, x)
    return np.ascontiguousarray(x.reshape(-1, W.shape[0]))


def _bipartite_problem(v0, v1, M, names):
    _vector(names[0], v0)
    _vector(names[1], v1)
    if len(M.shape) != 2:
        raise RuntimeError("wrong shape dim=(%s) = %s" % (names[2], M.shape))
    if v0.shape[0] != M.shape[1] or v1.shape[0] != M.shape[0]:
        _dims(", ".join(names), v0, v1, M)


def _bipartite_rows(W, a0, a1, caption, same_batch=True):
    _bits(a0, a1)
    if a0.shape[-1] != W.shape[1] or a1.shape[-1] != W.shape[0]:
        _dims(caption, a0, a1)
    a0 = np.ascontiguousarray(a0.reshape(-1, W.shape[1]))
    a1 = np.ascontiguousarray(a1.reshape(-1, W.shape[0]))
    if same_batch and a0.shape[0] != a1.shape[0]:
        raise RuntimeError("Different batch dims between x0 and x1.")
    return a0, a1


# ------------------------------------------------------------------- dense graph

def dense_graph_calculate_E(W, x, dtype):
    """QUBO energy x W x^T of one bit vector."""
    return dense_graph_batch_calculate_E(W, x, dtype)[0]


def dense_graph_batch_calculate_E(W, x, dtype):
    """QUBO energies of the rows of x (1-D x is one row)."""
    dtype = _check_dtype(dtype)
    W = common.fix_type(W, dtype)
    _square('W', W)
    W = common.symmetrize(W)
    x = _dense_rows(W, common.fix_type(x, np.int8), 'W, x')
    E = np.empty(x.shape[0], np.float64)
    _dg(dtype)('calculate_E', ptr(W), _c_int(W.shape[0]), ptr(x), _c_int(x.shape[0]), ptr(E))
    return E.astype(dtype)


def dense_graph_calculate_hamiltonian(W, dtype):
    """h, J, c of the Ising model of W (E_qubo(x) = E_ising(2 x - 1))."""
    dtype = _check_dtype(dtype)
    W = common.fix_type(W, dtype)
    _square('W', W)
    W = common.symmetrize(W)
    N = W.shape[0]
    h = np.empty(N, dtype)
    J = np.empty((N, N), dtype)
    c = np.empty(1, dtype)
    _dg(dtype)('calculate_hamiltonian', ptr(W), _c_int(N), ptr(h), ptr(J), ptr(c))
    return h, J, c[0]


def dense_graph_calculate_E_from_spin(h, J, c, q, dtype):
    """Ising energy -c - h q^T - q J q^T of one spin vector."""
    return dense_graph_batch_calculate_E_from_spin(h, J, c, common.fix_type(q, np.int8), dtype)[0]


def dense_graph_batch_calculate_E_from_spin(h, J, c, q, dtype):
    """Ising energies of the rows of q (1-D q is one row)."""
    dtype = _check_dtype(dtype)
    h, J = common.fix_type([h, J], dtype)
    _vector('h', h)
    _square('J', J)
    J = common.symmetrize(J)
    _scalar('c', c)
    if h.shape[0] != J.shape[0]:
        _dims('h, J', h, J)
    q = _dense_rows(J, q, 'J, q')
    E = np.empty(q.shape[0], np.float64)
    _dg(dtype)('calculate_E_from_spin', ptr(h), ptr(J), _real(dtype)(float(c)), _c_int(J.shape[0]),
               ptr(q), _c_int(q.shape[0]), ptr(E))
    return E.astype(dtype)


# --------------------------------------------------------------- bipartite graph

def bipartite_graph_calculate_E(b0, b1, W, x0, x1, dtype):
    """QUBO energy b0 x0^T + b1 x1^T + x1 W x0^T of one pair of bit vectors."""
    return bipartite_graph_batch_calculate_E(b0, b1, W, common.fix_type(x0, np.int8),
                                             common.fix_type(x1, np.int8), dtype)[0]


def bipartite_graph_batch_calculate_E(b0, b1, W, x0, x1, dtype):
    """QUBO energies of the row pairs (x0[i], x1[i])."""
    dtype = _check_dtype(dtype)
    b0, b1, W = common.fix_type([b0, b1, W], dtype)
    _bipartite_problem(b0, b1, W, ('b0', 'b1', 'W'))
    x0, x1 = _bipartite_rows(W, x0, x1, 'x0, x1')
    E = np.empty(x0.shape[0], np.float64)
    _bg(dtype)('calculate_E', ptr(b0), ptr(b1), ptr(W), _c_int(W.shape[1]), _c_int(W.shape[0]),
               ptr(x0), ptr(x1), _c_int(x0.shape[0]), ptr(E))
    return E.astype(dtype)


def bipartite_graph_batch_calculate_E_2d(b0, b1, W, x0, x1, dtype):
    """E[i1][i0]: the QUBO energy of every combination of a row of x1 and a row of x0."""
    dtype = _check_dtype(dtype)
    b0, b1, W = common.fix_type([b0, b1, W], dtype)
    x0, x1 = common.fix_type([x0, x1], np.int8)
    _bipartite_problem(b0, b1, W, ('b0', 'b1', 'W'))
    x0, x1 = _bipartite_rows(W, x0, x1, 'x0, x1', same_batch=False)
    m0, m1 = x0.shape[0], x1.shape[0]
    E = np.empty((m1, m0), np.float64)
    _bg(dtype)('calculate_E_2d', ptr(b0), ptr(b1), ptr(W), _c_int(W.shape[1]), _c_int(W.shape[0]),
               ptr(x0), _c_int(m0), ptr(x1), _c_int(m1), ptr(E))
    return E.astype(dtype)


def bipartite_graph_calculate_hamiltonian(b0, b1, W, dtype):
    """h0, h1, J, c of the Ising model of the bipartite QUBO (b0, b1, W)."""
    dtype = _check_dtype(dtype)
    b0, b1, W = common.fix_type([b0, b1, W], dtype)
    _bipartite_problem(b0, b1, W, ('b0', 'b1', 'W'))
    N1, N0 = W.shape
    h0 = np.empty(N0, dtype)
    h1 = np.empty(N1, dtype)
    J = np.empty((N1, N0), dtype)
    c = np.empty(1, dtype)
    _bg(dtype)('calculate_hamiltonian', ptr(b0), ptr(b1), ptr(W), _c_int(N0), _c_int(N1), ptr(h0),
               ptr(h1), ptr(J), ptr(c))
    return h0, h1, J, c[0]


def bipartite_graph_calculate_E_from_spin(h0, h1, J, c, q0, q1, dtype):
    """Ising energy -c - h0 q0^T - h1 q1^T - q1 J q0^T of one pair of spin vectors."""
    return bipartite_graph_batch_calculate_E_from_spin(h0, h1, J, c, common.fix_type(q0, np.int8),
                                                       common.fix_type(q1, np.int8), dtype)[0]


def bipartite_graph_batch_calculate_E_from_spin(h0, h1, J, c, q0, q1, dtype):
    """Ising energies of the row pairs (q0[i], q1[i])."""
    dtype = _check_dtype(dtype)
    h0, h1, J = common.fix_type([h0, h1, J], dtype)
    q0, q1 = common.fix_type([q0, q1], np.int8)
    _bipartite_problem(h0, h1, J, ('h0', 'h1', 'J'))
    _scalar('c', c)
    q0, q1 = _bipartite_rows(J, q0, q1, 'q0, q1')
    E = np.empty(q0.shape[0], np.float64)
    _bg(dtype)('calculate_E_from_spin', ptr(h0), ptr(h1), ptr(J), _real(dtype)(float(c)),
               _c_int(J.shape[1]), _c_int(J.shape[0]), ptr(q0), ptr(q1), _c_int(q0.shape[0]),
               ptr(E))
    return E.astype(dtype)
