"""cuda_dg_bf_searcher: the method table of sqaodc/pyglue/bf_searcher.inc:479-494
(DENSE_GRAPH, CUDA_SOLVER) on the dense-graph brute-force searchers of
libsqaod_gb300.so.  search_range returns (done, x) with x the next packed state
to search, as bf_searcher.inc:408-424 does."""
from ..cuda.solvers import DenseGraphBFSearcher
from . import _glue, cuda_device


def _bf(obj):
    return _glue.check_handle(obj, DenseGraphBFSearcher)


def new(dtype):
    return DenseGraphBFSearcher(None, None, _glue.check_dtype(dtype), None)


def delete(obj, dtype):
    _bf(obj).__del__()


def assign_device(obj, devobj, dtype):
    _bf(obj)
    cuda_device.assign(devobj)


def set_qubo(obj, W, optimize, dtype):
    _bf(obj).set_qubo(W, optimize)


def get_problem_size(obj, dtype):
    return _bf(obj).get_problem_size()


def set_preferences(obj, prefs, dtype):
    _bf(obj).set_preferences(prefs)


def get_preferences(obj, dtype):
    return _bf(obj).get_preferences()


def get_x(obj, dtype):
    return _bf(obj).get_x()


def get_E(obj, dtype):
    return _glue.to_E(_bf(obj).get_E(), _glue.check_dtype(dtype))


def prepare(obj, dtype):
    _bf(obj).prepare()


def calculate_E(obj, dtype):
    _bf(obj).calculate_E()


def make_solution(obj, dtype):
    _bf(obj).make_solution()


def search_range(obj, dtype):
    return _bf(obj).search_range_state()


def search(obj, dtype):
    _bf(obj).search()
