"""cuda_dg_annealer: the method table of sqaodc/pyglue/annealer.inc:885-908
(DENSE_GRAPH, CUDA_SOLVER) on the dense-graph annealers of libsqaod_gb300.so."""
import numpy as np

from ..cuda.solvers import DenseGraphAnnealer
from . import _glue, cuda_device


def _ann(obj):
    return _glue.check_handle(obj, DenseGraphAnnealer)


def new(dtype):
    return DenseGraphAnnealer(None, None, _glue.check_dtype(dtype), None)


def delete(obj, dtype):
    _ann(obj).__del__()


def assign_device(obj, devobj, dtype):
    _ann(obj)
    cuda_device.assign(devobj)


def seed(obj, seed, dtype):
    _ann(obj).seed(seed)


def set_qubo(obj, W, optimize, dtype):
    _ann(obj).set_qubo(W, optimize)


def set_hamiltonian(obj, h, J, c, dtype):
    _ann(obj).set_hamiltonian(h, J, c)


def get_problem_size(obj, dtype):
    return _ann(obj).get_problem_size()


def set_preferences(obj, prefs, dtype):
    _ann(obj).set_preferences(prefs)


def get_preferences(obj, dtype):
    return _ann(obj).get_preferences()


def get_E(obj, dtype):
    return _glue.to_E(_ann(obj).get_E(), _glue.check_dtype(dtype))


def get_x(obj, dtype):
    return _ann(obj).get_x()


def get_hamiltonian(obj, h, J, c, dtype):
    h1, J1, c1 = _ann(obj).get_hamiltonian()
    h[...] = h1
    J[...] = J1
    c[0] = c1


def get_q(obj, dtype):
    return _ann(obj).get_q()


def set_q(obj, q, dtype):
    if not isinstance(q, np.ndarray):
        raise RuntimeError("q is not an Array object.")
    _ann(obj).set_q(q)


def set_qset(obj, qset, dtype):
    _ann(obj).set_qset(qset)


def randomize_spin(obj, dtype):
    _ann(obj).randomize_spin()


def calculate_E(obj, dtype):
    _ann(obj).calculate_E()


def prepare(obj, dtype):
    _ann(obj).prepare()


def make_solution(obj, dtype):
    _ann(obj).make_solution()


def get_system_E(obj, G, beta, dtype):
    return _glue.check_dtype(dtype)(_ann(obj).get_system_E(G, beta))


def anneal_one_step(obj, G, beta, dtype):
    _ann(obj).anneal_one_step(G, beta)
