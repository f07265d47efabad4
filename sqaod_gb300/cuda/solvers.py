"""CUDA solvers of the sqaod Python API on libsqaod_gb300.so.

Same classes, factory functions, method names and argument meanings as
sqaodpy/sqaod/cuda/{dense_graph_annealer,bipartite_graph_annealer,
dense_graph_bf_searcher,bipartite_graph_bf_searcher}.py over the base
classes of sqaodpy/sqaod/common/*_base.py.  Every method forwards to one
handle-layer entry point of the C ABI (include/sqaod_gb300.h).

Every solver takes dtype numpy.float32 or numpy.float64 (the reference's
<double> instantiations: FP64 couplings, FP64 energies and minima; the
annealers' sweeps run on the fp32 rounding of the couplings and decide every
flagged trial from the FP64 ones); other dtypes raise.  The factories here
default to float32; the reference's default to float64 and pass the dtype on,
so code written against the reference gets the <double> solvers.
"""
import ctypes

import numpy as np

from .. import common
from .._lib import call, lib, ptr

_c_int = ctypes.c_int
_c_float = ctypes.c_float


def _check_dtype(dtype):
    d = np.dtype(np.float32 if dtype is None else dtype)
    if d not in (np.float32, np.float64):
        raise RuntimeError("dtype %s is not provided: the solvers compute in float32 or float64." % d)
    return d.type


def _pref_value(v):
    if isinstance(v, bool):
        return str(int(v))
    return str(v)


def _parse_prefs(s):
    out = {}
    for item in s.split(';'):
        if not item:
            continue
        k, v = item.split('=', 1)
        if k in ('n_trotters', 'tile_size', 'tile_size_0', 'tile_size_1'):
            v = int(v)
        out[k] = v
    return out


def _check_bf_dtype(dtype):
    """The brute-force searchers come in float32 and float64 (the <double> searchers)."""
    d = np.dtype(np.float32 if dtype is None else dtype)
    if d not in (np.float32, np.float64):
        raise RuntimeError("dtype %s is not provided: the searchers compute in float32 or float64." % d)
    return d.type


class _Handle:
    _prefix = None

    def __init__(self, new_name=None):
        self._L = lib()
        h = ctypes.c_void_p()
        call(getattr(self._L, new_name) if new_name else self._fn('new'), ctypes.byref(h))
        self._h = h

    def _fn(self, name):
        return getattr(self._L, '%s_%s' % (self._prefix, name))

    def _call(self, name, *args):
        return call(self._fn(name), self._h, *args)

    def __del__(self):
        h = getattr(self, '_h', None)
        if h is not None and h.value:
            try:
                self._fn('delete')(h)
            except Exception:
                pass
            self._h = None

    def set_preferences(self, prefdict=None, **prefs):
        merged = {}
        if prefdict is not None:
            merged.update(prefdict)
        merged.update(prefs)
        for k, v in merged.items():
            self._call('set_preference', str(k).encode(), _pref_value(v).encode())

    def get_preferences(self):
        buf = ctypes.create_string_buffer(512)
        self._call('get_preferences', buf, _c_int(512))
        return _parse_prefs(buf.value.decode())

    def get_optimize_dir(self):
        return self._optimize


class DenseGraphAnnealer(_Handle):
    """Dense-graph annealer (sqaodpy/sqaod/common/dense_graph_annealer_base.py)."""
    _prefix = 'sq103_dg_annealer'

    def __init__(self, W, optimize, dtype, prefdict):
        self.dtype = _check_dtype(dtype)
        self._f64 = self.dtype is np.float64
        super().__init__('sq103_dg_annealer64_new' if self._f64 else None)
        self._optimize = common.minimize
        if W is not None:
            self.set_qubo(W, optimize)
        self.set_preferences(prefdict)

    def seed(self, seed):
        self._call('seed', ctypes.c_ulonglong(int(seed)))

    def set_qubo(self, W, optimize=common.minimize):
        common.check_square(W)
        W = common.fix_type(W, self.dtype)
        om = _c_int(common.optimize_flag(optimize))
        fn = 'set_qubo64' if self._f64 else 'set_qubo'
        common.submit_symmetric(W, self.dtype, lambda w: self._call(fn, ptr(w), _c_int(w.shape[0]), om))
        self._optimize = optimize

    def set_hamiltonian(self, h, J, c):
        common.check_square(J, 'J')
        h, J = common.fix_type([np.asarray(h), np.asarray(J)], self.dtype)
        J = np.ascontiguousarray(common.symmetrize(J), self.dtype)
        if self._f64:
            self._call('set_hamiltonian64', ptr(h), ptr(J), ctypes.c_double(float(c)), _c_int(J.shape[0]))
        else:
            self._call('set_hamiltonian', ptr(h), ptr(J), _c_float(float(c)), _c_int(J.shape[0]))
        self._optimize = common.minimize

    def get_problem_size(self):
        n = _c_int()
        self._call('get_problem_size', ctypes.byref(n))
        return n.value

    def _m(self):
        return self.get_preferences()['n_trotters']

    def get_E(self):
        if self._f64:
            return self.get_E64()
        cap = max(self._m(), 1)
        E = np.zeros(cap, np.float32)
        n = _c_int()
        self._call('get_E', ptr(E), _c_int(cap), ctypes.byref(n))
        return E[:n.value].copy()

    def get_E64(self):
        """FP64 energies of the trotters (extension)."""
        cap = max(self._m(), 1)
        E = np.zeros(cap, np.float64)
        n = _c_int()
        self._call('get_E64', ptr(E), _c_int(cap), ctypes.byref(n))
        return E[:n.value].copy()

    def calculate_E(self):
        self._call('calculate_E')

    def _bits(self, name):
        N, m = self.get_problem_size(), max(self._m(), 1)
        out = np.zeros((m, N), np.int8)
        n = _c_int()
        self._call(name, ptr(out), _c_int(m), ctypes.byref(n))
        return [out[i].copy() for i in range(n.value)]

    def get_x(self):
        return self._bits('get_x')

    def get_q(self):
        return self._bits('get_q')

    def set_q(self, q):
        q = np.ascontiguousarray(common.fix_type(np.asarray(q), np.int8)).ravel()
        self._call('set_q', ptr(q), _c_int(len(q)))

    def set_qset(self, qset):
        qs = np.ascontiguousarray(np.array([common.fix_type(np.asarray(v), np.int8) for v in qset]), np.int8)
        self._call('set_qset', ptr(qs), _c_int(qs.shape[0]), _c_int(qs.shape[1]))

    def get_hamiltonian(self):
        N = self.get_problem_size()
        h = np.empty(N, self.dtype)
        J = np.empty((N, N), self.dtype)
        c = np.empty(1, self.dtype)
        self._call('get_hamiltonian64' if self._f64 else 'get_hamiltonian', ptr(h), ptr(J), ptr(c))
        return h, J, c[0]

    def randomize_spin(self):
        self._call('randomize_spin')

    def prepare(self):
        self._call('prepare')

    def init_anneal(self):
        """prepare() + randomize_spin()."""
        self._call('init_anneal')

    def make_solution(self):
        self._call('make_solution')

    def get_system_E(self, G, beta):
        if self._f64:
            E = ctypes.c_double()
            self._call('get_system_E64', ctypes.c_double(G), ctypes.c_double(beta), ctypes.byref(E))
            return np.float64(E.value)
        E = _c_float()
        self._call('get_system_E', _c_float(G), _c_float(beta), ctypes.byref(E))
        return np.float32(E.value)

    def anneal_one_step(self, G, beta):
        self._call('anneal_one_step', _c_float(G), _c_float(beta))

    def anneal(self, G, beta):
        """Runs len(G) annealOneStep steps in one call (extension)."""
        G = np.ascontiguousarray(G, np.float32)
        beta = np.ascontiguousarray(np.broadcast_to(np.asarray(beta, np.float32), G.shape), np.float32)
        self._call('anneal', ptr(G), ptr(beta), _c_int(len(G)))

    def get_accepted(self):
        v = ctypes.c_ulonglong()
        self._call('get_accepted', ctypes.byref(v))
        return v.value

    def get_rng_state(self):
        s, st = ctypes.c_ulonglong(), ctypes.c_uint32()
        self._call('get_rng_state', ctypes.byref(s), ctypes.byref(st))
        return s.value, st.value

    def get_checkpoint(self):
        """The annealing state as a dict of numpy values (numpy.savez stores it):
        spins q (m x N int8), resident local fields F (m x N float32), the Philox
        seed and step counter, and the steps since the last field refresh.
        No counterpart in the reference."""
        N, m = self.get_problem_size(), self._m()
        q = np.empty((m, N), np.int8)
        F = np.empty((m, N), np.float32)
        s, st, since = ctypes.c_ulonglong(), ctypes.c_uint32(), ctypes.c_int()
        self._call('get_checkpoint', ptr(q), ptr(F), ctypes.byref(s), ctypes.byref(st), ctypes.byref(since))
        return {'q': q, 'F': F, 'seed': np.uint64(s.value), 'step': np.uint32(st.value),
                'since_refresh': np.int32(since.value)}

    def set_checkpoint(self, state):
        """Restores get_checkpoint()'s state into this prepared annealer (same
        problem, algorithm and n_trotters): annealing then continues bit for bit
        as in the annealer the state was taken from."""
        q = np.ascontiguousarray(state['q'], np.int8)
        F = np.ascontiguousarray(state['F'], np.float32)
        if q.ndim != 2 or F.shape != q.shape:
            raise RuntimeError("checkpoint q and F must be matrices of the same shape.")
        self._call('set_checkpoint', ptr(q), ptr(F), _c_int(q.shape[0]), _c_int(q.shape[1]),
                   ctypes.c_ulonglong(int(state['seed'])), ctypes.c_uint32(int(state['step'])),
                   _c_int(int(state['since_refresh'])))

    def set_trace(self, enable):
        self._call('set_trace', _c_int(1 if enable else 0))

    def get_trace(self, nwords):
        out = np.zeros(nwords, np.uint32)
        self._call('get_trace', ptr(out), _c_int(nwords))
        return out

    def set_kernel(self, flags):
        """Sweep kernel: 0 automatic, 1 one CTA per instance, 2 one CTA per trotter (extension)."""
        self._call('set_kernel', _c_int(flags))


class BipartiteGraphAnnealer(_Handle):
    """Bipartite-graph annealer (sqaodpy/sqaod/common/bipartite_graph_annealer_base.py)."""
    _prefix = 'sq103_bg_annealer'

    def __init__(self, b0, b1, W, optimize, dtype, prefdict):
        self.dtype = _check_dtype(dtype)
        self._f64 = self.dtype is np.float64
        super().__init__('sq103_bg_annealer64_new' if self._f64 else None)
        self._optimize = common.minimize
        if W is not None:
            self.set_qubo(b0, b1, W, optimize)
        self.set_preferences(prefdict)

    def seed(self, seed):
        self._call('seed', ctypes.c_ulonglong(int(seed)))

    def set_qubo(self, b0, b1, W, optimize=common.minimize):
        b0, b1, W = common.fix_type([np.asarray(b0), np.asarray(b1), np.asarray(W)], self.dtype)
        if W.ndim != 2 or W.shape != (len(b1), len(b0)):
            raise RuntimeError('dimension mismatch for b0, b1, W.')
        self._call('set_qubo64' if self._f64 else 'set_qubo', ptr(b0), ptr(b1), ptr(W), _c_int(len(b0)),
                   _c_int(len(b1)), _c_int(common.optimize_flag(optimize)))
        self._optimize = optimize

    def set_hamiltonian(self, h0, h1, J, c):
        h0, h1, J = common.fix_type([np.asarray(h0), np.asarray(h1), np.asarray(J)], self.dtype)
        if J.ndim != 2 or J.shape != (len(h1), len(h0)):
            raise RuntimeError('dimension mismatch for h0, h1, J.')
        if self._f64:
            self._call('set_hamiltonian64', ptr(h0), ptr(h1), ptr(J), ctypes.c_double(float(c)), _c_int(len(h0)),
                       _c_int(len(h1)))
        else:
            self._call('set_hamiltonian', ptr(h0), ptr(h1), ptr(J), _c_float(float(c)), _c_int(len(h0)),
                       _c_int(len(h1)))
        self._optimize = common.minimize

    def get_problem_size(self):
        a, b = _c_int(), _c_int()
        self._call('get_problem_size', ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def _m(self):
        return self.get_preferences()['n_trotters']

    def get_E(self):
        if self._f64:
            return self.get_E64()
        cap = max(self._m(), 1)
        E = np.zeros(cap, np.float32)
        n = _c_int()
        self._call('get_E', ptr(E), _c_int(cap), ctypes.byref(n))
        return E[:n.value].copy()

    def get_E64(self):
        cap = max(self._m(), 1)
        E = np.zeros(cap, np.float64)
        n = _c_int()
        self._call('get_E64', ptr(E), _c_int(cap), ctypes.byref(n))
        return E[:n.value].copy()

    def calculate_E(self):
        self._call('calculate_E')

    def _pairs(self, name):
        (N0, N1), m = self.get_problem_size(), max(self._m(), 1)
        a = np.zeros((m, N0), np.int8)
        b = np.zeros((m, N1), np.int8)
        n = _c_int()
        self._call(name, ptr(a), ptr(b), _c_int(m), ctypes.byref(n))
        return [(a[i].copy(), b[i].copy()) for i in range(n.value)]

    def get_x(self):
        return self._pairs('get_x')

    def get_q(self):
        return self._pairs('get_q')

    def set_q(self, qpair):
        # any shape with N0 (N1) elements, e.g. the (1, N) rows of bit_to_spin, as the reference takes them
        q0, q1 = (np.ascontiguousarray(common.fix_type(np.asarray(v), np.int8)).ravel() for v in qpair)
        self._call('set_q', ptr(q0), ptr(q1), _c_int(len(q0)), _c_int(len(q1)))

    def set_qset(self, qset):
        q0 = np.ascontiguousarray(np.array([np.asarray(p[0], np.int8) for p in qset]), np.int8)
        q1 = np.ascontiguousarray(np.array([np.asarray(p[1], np.int8) for p in qset]), np.int8)
        self._call('set_qset', ptr(q0), ptr(q1), _c_int(q0.shape[0]), _c_int(q0.shape[1]), _c_int(q1.shape[1]))

    def get_hamiltonian(self):
        N0, N1 = self.get_problem_size()
        h0 = np.empty(N0, self.dtype)
        h1 = np.empty(N1, self.dtype)
        J = np.empty((N1, N0), self.dtype)
        c = np.empty(1, self.dtype)
        self._call('get_hamiltonian64' if self._f64 else 'get_hamiltonian', ptr(h0), ptr(h1), ptr(J), ptr(c))
        return h0, h1, J, c[0]

    def randomize_spin(self):
        self._call('randomize_spin')

    def prepare(self):
        self._call('prepare')

    def init_anneal(self):
        self._call('init_anneal')

    def make_solution(self):
        self._call('make_solution')

    def get_system_E(self, G, beta):
        if self._f64:
            E = ctypes.c_double()
            self._call('get_system_E64', ctypes.c_double(G), ctypes.c_double(beta), ctypes.byref(E))
            return np.float64(E.value)
        E = _c_float()
        self._call('get_system_E', _c_float(G), _c_float(beta), ctypes.byref(E))
        return np.float32(E.value)

    def anneal_one_step(self, G, beta):
        self._call('anneal_one_step', _c_float(G), _c_float(beta))

    def anneal(self, G, beta):
        G = np.ascontiguousarray(G, np.float32)
        beta = np.ascontiguousarray(np.broadcast_to(np.asarray(beta, np.float32), G.shape), np.float32)
        self._call('anneal', ptr(G), ptr(beta), _c_int(len(G)))

    def get_accepted(self):
        v = ctypes.c_ulonglong()
        self._call('get_accepted', ctypes.byref(v))
        return v.value

    def get_rng_state(self):
        s, st = ctypes.c_ulonglong(), ctypes.c_uint32()
        self._call('get_rng_state', ctypes.byref(s), ctypes.byref(st))
        return s.value, st.value

    def get_checkpoint(self):
        """The annealing state as a dict of numpy values (numpy.savez stores it):
        spins q0 (m x N0) and q1 (m x N1), int8, and the Philox seed and step
        counter.  No counterpart in the reference."""
        N0, N1 = self.get_problem_size()
        m = self._m()
        q0 = np.empty((m, N0), np.int8)
        q1 = np.empty((m, N1), np.int8)
        s, st = ctypes.c_ulonglong(), ctypes.c_uint32()
        self._call('get_checkpoint', ptr(q0), ptr(q1), ctypes.byref(s), ctypes.byref(st))
        return {'q0': q0, 'q1': q1, 'seed': np.uint64(s.value), 'step': np.uint32(st.value)}

    def set_checkpoint(self, state):
        """Restores get_checkpoint()'s state into this prepared annealer (same
        problem, algorithm and n_trotters); annealing continues bit for bit."""
        q0 = np.ascontiguousarray(state['q0'], np.int8)
        q1 = np.ascontiguousarray(state['q1'], np.int8)
        if q0.ndim != 2 or q1.ndim != 2 or q0.shape[0] != q1.shape[0]:
            raise RuntimeError("checkpoint q0 and q1 must be matrices with the same number of rows.")
        self._call('set_checkpoint', ptr(q0), ptr(q1), _c_int(q0.shape[0]), _c_int(q0.shape[1]),
                   _c_int(q1.shape[1]), ctypes.c_ulonglong(int(state['seed'])),
                   ctypes.c_uint32(int(state['step'])))

    def set_trace(self, enable):
        self._call('set_trace', _c_int(1 if enable else 0))

    def get_trace(self, nwords):
        out = np.zeros(nwords, np.uint32)
        self._call('get_trace', ptr(out), _c_int(nwords))
        return out


class DenseGraphBFSearcher(_Handle):
    """Dense-graph brute-force searcher (sqaodpy/sqaod/common/dense_graph_bf_searcher_base.py)."""
    _prefix = 'sq103_dg_bf'

    def __init__(self, W, optimize, dtype, prefdict):
        self.dtype = _check_bf_dtype(dtype)
        super().__init__('sq103_dg_bf64_new' if self.dtype is np.float64 else None)
        self._optimize = common.minimize
        if W is not None:
            self.set_qubo(W, optimize)
        self.set_preferences(prefdict)

    def set_qubo(self, W, optimize=common.minimize):
        common.check_square(W)
        W = common.fix_type(W, self.dtype)
        om = _c_int(common.optimize_flag(optimize))
        fn = 'set_qubo64' if self.dtype is np.float64 else 'set_qubo'
        common.submit_symmetric(W, self.dtype, lambda w: self._call(fn, ptr(w), _c_int(w.shape[0]), om))
        self._optimize = optimize

    def get_problem_size(self):
        n = _c_int()
        self._call('get_problem_size', ctypes.byref(n))
        return n.value

    def _cap(self):
        return max(self.get_preferences()['tile_size'], 1)

    def get_E(self):
        cap = self._cap()
        E = np.zeros(cap, np.float32)
        n = _c_int()
        self._call('get_E', ptr(E), _c_int(cap), ctypes.byref(n))
        if self.dtype is np.float64:  # every solution has the exact FP64 minimum
            return np.full(n.value, self.get_E64(), np.float64)
        return E[:n.value].copy()

    def get_x(self):
        N, cap = self.get_problem_size(), self._cap()
        out = np.zeros((cap, N), np.int8)
        n = _c_int()
        self._call('get_x', ptr(out), _c_int(cap), ctypes.byref(n))
        return [out[i].copy() for i in range(n.value)]

    def prepare(self):
        self._call('prepare')

    def calculate_E(self):
        self._call('calculate_E')

    def make_solution(self):
        self._call('make_solution')

    def search_range(self):
        return self.search_range_state()[0]

    def search_range_state(self):
        """One searchRange step: (done, x) with x the next packed state to search
        (the reference extension's return value, sqaodc/pyglue/bf_searcher.inc:408-424)."""
        x = ctypes.c_ulonglong()
        done = _c_int()
        self._call('search_range', ctypes.byref(x), ctypes.byref(done))
        return bool(done.value), x.value

    def search(self):
        self._call('search')

    def search_subrange(self, x_begin, x_end):
        """Searches the packed states [x_begin, x_end) after prepare() (one shard of
        a multi-GPU search; the ranges given to one searcher must ascend).  No
        counterpart in the reference."""
        self._call('search_subrange', ctypes.c_ulonglong(int(x_begin)), ctypes.c_ulonglong(int(x_end)))

    def get_E64(self):
        """Exact FP64 minimum found so far (negated for maximize)."""
        e = ctypes.c_double()
        self._call('get_E64', ctypes.byref(e))
        return e.value


class BipartiteGraphBFSearcher(_Handle):
    """Bipartite-graph brute-force searcher (sqaodpy/sqaod/common/bipartite_graph_bf_searcher_base.py)."""
    _prefix = 'sq103_bg_bf'

    def __init__(self, b0, b1, W, optimize, dtype, prefdict):
        self.dtype = _check_bf_dtype(dtype)
        super().__init__('sq103_bg_bf64_new' if self.dtype is np.float64 else None)
        self._optimize = common.minimize
        if W is not None:
            self.set_qubo(b0, b1, W, optimize)
        self.set_preferences(prefdict)

    def set_qubo(self, b0, b1, W, optimize=common.minimize):
        b0, b1, W = common.fix_type([np.asarray(b0), np.asarray(b1), np.asarray(W)], self.dtype)
        if W.ndim != 2 or W.shape != (len(b1), len(b0)):
            raise RuntimeError('dimension mismatch for b0, b1, W.')
        self._call('set_qubo64' if self.dtype is np.float64 else 'set_qubo', ptr(b0), ptr(b1), ptr(W),
                   _c_int(len(b0)), _c_int(len(b1)), _c_int(common.optimize_flag(optimize)))
        self._optimize = optimize

    def get_problem_size(self):
        a, b = _c_int(), _c_int()
        self._call('get_problem_size', ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def _cap(self):
        p = self.get_preferences()
        return max(p['tile_size_0'] + p['tile_size_1'], 1)

    def get_E(self):
        cap = self._cap()
        E = np.zeros(cap, np.float32)
        n = _c_int()
        self._call('get_E', ptr(E), _c_int(cap), ctypes.byref(n))
        if self.dtype is np.float64:  # every solution has the exact FP64 minimum
            return np.full(n.value, self.get_E64(), np.float64)
        return E[:n.value].copy()

    def get_x(self):
        (N0, N1), cap = self.get_problem_size(), self._cap()
        a = np.zeros((cap, N0), np.int8)
        b = np.zeros((cap, N1), np.int8)
        n = _c_int()
        self._call('get_x', ptr(a), ptr(b), _c_int(cap), ctypes.byref(n))
        return [(a[i].copy(), b[i].copy()) for i in range(n.value)]

    def prepare(self):
        self._call('prepare')

    def calculate_E(self):
        self._call('calculate_E')

    def make_solution(self):
        self._call('make_solution')

    def search_range(self):
        return self.search_range_state()[0]

    def search_range_state(self):
        """One searchRange step: (done, x0, x1), the next packed states to search
        (sqaodc/pyglue/bf_searcher.inc:432-448)."""
        x0, x1 = ctypes.c_ulonglong(), ctypes.c_ulonglong()
        done = _c_int()
        self._call('search_range', ctypes.byref(x0), ctypes.byref(x1), ctypes.byref(done))
        return bool(done.value), x0.value, x1.value

    def search(self):
        self._call('search')

    def get_E64(self):
        """Exact FP64 minimum found so far (negated for maximize)."""
        e = ctypes.c_double()
        self._call('get_E64', ctypes.byref(e))
        return e.value


def dense_graph_annealer(W=None, optimize=common.minimize, dtype=np.float32, **prefs):
    """Factory of DenseGraphAnnealer (sqaodpy/sqaod/cuda/dense_graph_annealer.py:18-31)."""
    return DenseGraphAnnealer(W, optimize, dtype, prefs)


def bipartite_graph_annealer(b0=None, b1=None, W=None, optimize=common.minimize, dtype=np.float32, **prefs):
    """Factory of BipartiteGraphAnnealer (sqaodpy/sqaod/cuda/bipartite_graph_annealer.py)."""
    return BipartiteGraphAnnealer(b0, b1, W, optimize, dtype, prefs)


def dense_graph_bf_searcher(W=None, optimize=common.minimize, dtype=np.float32, **prefs):
    """Factory of DenseGraphBFSearcher (sqaodpy/sqaod/cuda/dense_graph_bf_searcher.py)."""
    return DenseGraphBFSearcher(W, optimize, dtype, prefs)


def bipartite_graph_bf_searcher(b0=None, b1=None, W=None, optimize=common.minimize, dtype=np.float32, **prefs):
    """Factory of BipartiteGraphBFSearcher (sqaodpy/sqaod/cuda/bipartite_graph_bf_searcher.py)."""
    return BipartiteGraphBFSearcher(b0, b1, W, optimize, dtype, prefs)
