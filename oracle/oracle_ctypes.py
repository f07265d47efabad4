"""ctypes bindings to the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference legs of bench.py.  The product package never imports
this module.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

ALGO_NAIVE, ALGO_COLORING, ALGO_SA_NAIVE, ALGO_SA_COLORING = 0, 1, 2, 3


class ReplayStats(ctypes.Structure):
    _fields_ = [("n_trials", ctypes.c_longlong), ("n_accept", ctypes.c_longlong),
                ("n_mismatch", ctypes.c_longlong), ("n_mismatch_small", ctypes.c_longlong),
                ("n_small_margin", ctypes.c_longlong), ("max_mismatch_margin", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib():
    global _lib
    if _lib is None:
        path = _build.oracle_lib_path()
        if not os.path.exists(path):
            _build.build_oracle()
        _lib = ctypes.CDLL(path)
        _lib.orc_dot_ref.restype = ctypes.c_float
        _lib.orc_mt_f32.restype = ctypes.c_float
        _lib.orc_dg_bf_sweep_tiles.restype = ctypes.c_float
        _lib.orc_dga_new.restype = ctypes.c_void_p
        _lib.orc_bga_new.restype = ctypes.c_void_p
        for f in ("orc_dga_free", "orc_dga_set_hamiltonian", "orc_dga_seed", "orc_dga_randomize",
                  "orc_dga_set_q", "orc_dga_get_q", "orc_dga_step", "orc_dga_energy",
                  "orc_dga_workers", "orc_bga_free", "orc_bga_set_hamiltonian", "orc_bga_seed",
                  "orc_bga_randomize", "orc_bga_set_q", "orc_bga_get_q", "orc_bga_step",
                  "orc_bga_energy"):
            getattr(_lib, f).argtypes = None
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, np.float64)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _i8(a):
    return np.ascontiguousarray(a, np.int8)


# ---------------------------------------------------------------- RNG
def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().orc_philox(_p(c), _p(k), _p(o))
    return o


def mt_stream(seed, n):
    out = np.zeros(n, np.uint32)
    lib().orc_mt_stream(ctypes.c_ulonglong(seed), ctypes.c_int(n), _p(out))
    return out


def dot_ref(a, b):
    n = len(a)
    pad = (n + 15) // 16 * 16
    pa = np.zeros(pad, np.float32)
    pb = np.zeros(pad, np.float32)
    pa[:n] = a
    pb[:n] = b
    return lib().orc_dot_ref(_p(pa), _p(pb), ctypes.c_int(n))


# ----------------------------------------------------------- formulas
def dg_hamiltonian(W):
    W = _f64(W)
    N = W.shape[0]
    h = np.zeros(N)
    J = np.zeros((N, N))
    c = np.zeros(1)
    lib().orc_dg_hamiltonian(_p(W), ctypes.c_int(N), _p(h), _p(J), _p(c))
    return h, J, c[0]


def dg_energy_qubo(W, x):
    W = _f64(W)
    x = _i8(np.atleast_2d(x))
    E = np.zeros(x.shape[0])
    lib().orc_dg_energy_qubo(_p(W), ctypes.c_int(W.shape[0]), _p(x), ctypes.c_int(x.shape[0]), _p(E))
    return E


def dg_energy_ising(h, J, c, q):
    h, J = _f64(h), _f64(J)
    q = _i8(np.atleast_2d(q))
    E = np.zeros(q.shape[0])
    lib().orc_dg_energy_ising(_p(h), _p(J), ctypes.c_double(c), ctypes.c_int(len(h)), _p(q),
                              ctypes.c_int(q.shape[0]), _p(E))
    return E


def bg_hamiltonian(b0, b1, W):
    b0, b1, W = _f64(b0), _f64(b1), _f64(W)
    N0, N1 = len(b0), len(b1)
    h0, h1, J, c = np.zeros(N0), np.zeros(N1), np.zeros((N1, N0)), np.zeros(1)
    lib().orc_bg_hamiltonian(_p(b0), _p(b1), _p(W), ctypes.c_int(N0), ctypes.c_int(N1),
                             _p(h0), _p(h1), _p(J), _p(c))
    return h0, h1, J, c[0]


def bg_energy_qubo(b0, b1, W, x0, x1):
    b0, b1, W = _f64(b0), _f64(b1), _f64(W)
    x0, x1 = _i8(np.atleast_2d(x0)), _i8(np.atleast_2d(x1))
    E = np.zeros(x0.shape[0])
    lib().orc_bg_energy_qubo(_p(b0), _p(b1), _p(W), ctypes.c_int(len(b0)), ctypes.c_int(len(b1)),
                             _p(x0), _p(x1), ctypes.c_int(x0.shape[0]), _p(E))
    return E


def bg_energy_qubo_2d(b0, b1, W, x0, x1):
    b0, b1, W = _f64(b0), _f64(b1), _f64(W)
    x0, x1 = _i8(np.atleast_2d(x0)), _i8(np.atleast_2d(x1))
    E = np.zeros((x1.shape[0], x0.shape[0]))
    lib().orc_bg_energy_qubo_2d(_p(b0), _p(b1), _p(W), ctypes.c_int(len(b0)), ctypes.c_int(len(b1)),
                                _p(x0), ctypes.c_int(x0.shape[0]), _p(x1), ctypes.c_int(x1.shape[0]),
                                _p(E))
    return E


def bg_energy_ising(h0, h1, J, c, q0, q1):
    h0, h1, J = _f64(h0), _f64(h1), _f64(J)
    q0, q1 = _i8(np.atleast_2d(q0)), _i8(np.atleast_2d(q1))
    E = np.zeros(q0.shape[0])
    lib().orc_bg_energy_ising(_p(h0), _p(h1), _p(J), ctypes.c_double(c), ctypes.c_int(len(h0)),
                              ctypes.c_int(len(h1)), _p(q0), _p(q1), ctypes.c_int(q0.shape[0]), _p(E))
    return E


# ------------------------------------------------------ BF searchers
def unpack_bits(packed, N):
    packed = np.asarray(packed, np.uint64)
    shifts = np.arange(N - 1, -1, -1, dtype=np.uint64)
    return ((packed[:, None] >> shifts[None, :]) & np.uint64(1)).astype(np.int8)


def dg_bf_search_ref(W, om=0, tile_size=1024, n_workers=0, cap=1 << 20):
    W = _f32(W)
    xs = np.zeros(cap, np.uint64)
    E = ctypes.c_float()
    n = lib().orc_dg_bf_search_ref(_p(W), ctypes.c_int(W.shape[0]), ctypes.c_int(om),
                                   ctypes.c_int(tile_size), ctypes.c_int(n_workers),
                                   ctypes.byref(E), _p(xs), ctypes.c_int(cap))
    return E.value, xs[:n].copy()


def dg_bf_search_exact_int(W, om=0, cap=1024, n_workers=0):
    """Exact integer search of every state in Gray-code order (integer-valued
    symmetric W only).  Returns (Emin, first `cap` minimisers ascending, count of
    minimisers)."""
    W = _f32(W)
    xs = np.zeros(max(cap, 1), np.uint64)
    E = ctypes.c_double()
    cnt = ctypes.c_longlong()
    n = lib().orc_dg_bf_search_exact_int(_p(W), ctypes.c_int(W.shape[0]), ctypes.c_int(om), ctypes.c_int(cap),
                                         ctypes.c_int(n_workers), ctypes.byref(E), _p(xs), ctypes.byref(cnt))
    if n < 0:
        raise ValueError("orc_dg_bf_search_exact_int failed (%d)" % n)
    return E.value, xs[:n].copy(), cnt.value


def dg_bf_search_range(W, om, x_begin, x_end, cap):
    W = _f32(W)
    xs = np.zeros(cap, np.uint64)
    E = ctypes.c_float()
    n = lib().orc_dg_bf_search_range(_p(W), ctypes.c_int(W.shape[0]), ctypes.c_int(om),
                                     ctypes.c_uint64(x_begin), ctypes.c_uint64(x_end),
                                     ctypes.c_int(cap), ctypes.byref(E), _p(xs))
    return E.value, xs[:n].copy()


def dg_bf_sweep_tiles(W, x_begin, tile_size, n_tiles, n_workers=0):
    W = _f32(W)
    return lib().orc_dg_bf_sweep_tiles(_p(W), ctypes.c_int(W.shape[0]), ctypes.c_uint64(x_begin),
                                       ctypes.c_int(tile_size), ctypes.c_int(n_tiles),
                                       ctypes.c_int(n_workers))


def bg_bf_search_ref(b0, b1, W, om=0, tile0=1024, tile1=1024, n_workers=0, cap=1 << 16):
    b0, b1, W = _f32(b0), _f32(b1), _f32(W)
    xs = np.zeros(2 * cap, np.uint64)
    E = ctypes.c_float()
    n = lib().orc_bg_bf_search_ref(_p(b0), _p(b1), _p(W), ctypes.c_int(len(b0)), ctypes.c_int(len(b1)),
                                   ctypes.c_int(om), ctypes.c_int(tile0), ctypes.c_int(tile1),
                                   ctypes.c_int(n_workers), ctypes.byref(E), _p(xs), ctypes.c_int(cap))
    return E.value, xs[:2 * n].reshape(-1, 2).copy()


def bg_bf_search_sorted(b0, b1, W, om=0, cap=1 << 16):
    b0, b1, W = _f32(b0), _f32(b1), _f32(W)
    xs = np.zeros(2 * cap, np.uint64)
    E = ctypes.c_float()
    n = lib().orc_bg_bf_search_sorted(_p(b0), _p(b1), _p(W), ctypes.c_int(len(b0)), ctypes.c_int(len(b1)),
                                      ctypes.c_int(om), ctypes.c_int(cap), ctypes.byref(E), _p(xs))
    return E.value, xs[:2 * n].reshape(-1, 2).copy()


# ------------------------------------------- reference CPU annealers
class DenseAnnealerRef:
    """The reference CPU dense annealer (sqaodc/cpu/CPUDenseGraphAnnealer.cpp)."""

    def __init__(self, h, J, c, m, n_workers=0):
        L = lib()
        self.N, self.m = len(h), m
        self._h = L.orc_dga_new(ctypes.c_int(self.N), ctypes.c_int(m), ctypes.c_int(n_workers))
        h, J = _f32(h), _f32(J)
        L.orc_dga_set_hamiltonian(ctypes.c_void_p(self._h), _p(h), _p(J), ctypes.c_float(c))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_dga_free(ctypes.c_void_p(self._h))
            self._h = None

    @property
    def workers(self):
        return lib().orc_dga_workers(ctypes.c_void_p(self._h))

    def seed(self, s):
        lib().orc_dga_seed(ctypes.c_void_p(self._h), ctypes.c_ulonglong(s))

    def randomize_spin(self):
        lib().orc_dga_randomize(ctypes.c_void_p(self._h))

    def set_q(self, q):
        q = _i8(q)
        lib().orc_dga_set_q(ctypes.c_void_p(self._h), _p(q))

    def get_q(self):
        q = np.zeros((self.m, self.N), np.int8)
        lib().orc_dga_get_q(ctypes.c_void_p(self._h), _p(q))
        return q

    def anneal_one_step(self, algo, G, beta):
        lib().orc_dga_step(ctypes.c_void_p(self._h), ctypes.c_int(algo), ctypes.c_float(G),
                           ctypes.c_float(beta))

    def get_E(self):
        E = np.zeros(self.m)
        lib().orc_dga_energy(ctypes.c_void_p(self._h), _p(E))
        return E


class BipartiteAnnealerRef:
    """The reference CPU bipartite annealer (sqaodc/cpu/CPUBipartiteGraphAnnealer.cpp)."""

    def __init__(self, h0, h1, J, c, m, n_workers=0):
        L = lib()
        self.N0, self.N1, self.m = len(h0), len(h1), m
        self._h = L.orc_bga_new(ctypes.c_int(self.N0), ctypes.c_int(self.N1), ctypes.c_int(m),
                                ctypes.c_int(n_workers))
        h0, h1, J = _f32(h0), _f32(h1), _f32(J)
        L.orc_bga_set_hamiltonian(ctypes.c_void_p(self._h), _p(h0), _p(h1), _p(J), ctypes.c_float(c))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_bga_free(ctypes.c_void_p(self._h))
            self._h = None

    @property
    def workers(self):
        return lib().orc_bga_workers(ctypes.c_void_p(self._h))

    def seed(self, s):
        lib().orc_bga_seed(ctypes.c_void_p(self._h), ctypes.c_ulonglong(s))

    def randomize_spin(self):
        lib().orc_bga_randomize(ctypes.c_void_p(self._h))

    def set_q(self, q0, q1):
        q0, q1 = _i8(q0), _i8(q1)
        lib().orc_bga_set_q(ctypes.c_void_p(self._h), _p(q0), _p(q1))

    def get_q(self):
        q0 = np.zeros((self.m, self.N0), np.int8)
        q1 = np.zeros((self.m, self.N1), np.int8)
        lib().orc_bga_get_q(ctypes.c_void_p(self._h), _p(q0), _p(q1))
        return q0, q1

    def anneal_one_step(self, algo, G, beta):
        lib().orc_bga_step(ctypes.c_void_p(self._h), ctypes.c_int(algo), ctypes.c_float(G),
                           ctypes.c_float(beta))

    def get_E(self):
        E = np.zeros(self.m)
        lib().orc_bga_energy(ctypes.c_void_p(self._h), _p(E))
        return E


# ------------------------------------------------------- FP64 replay
def gpu_randomize(seed, step, tag_side, m, N):
    q = np.zeros((m, N), np.int8)
    lib().orc_gpu_randomize(ctypes.c_uint64(seed), ctypes.c_uint32(step), ctypes.c_int(tag_side),
                            ctypes.c_int(m), ctypes.c_int(N), _p(q))
    return q


def dg_replay(h, J, m, algo, seed, step, G, beta, q, trace, tol=1e-6):
    h, J = _f32(h), _f32(J)
    q = _i8(q).copy()
    trace = np.ascontiguousarray(trace, np.uint32)
    st = ReplayStats()
    lib().orc_dg_replay(_p(h), _p(J), ctypes.c_int(len(h)), ctypes.c_int(m), ctypes.c_int(algo),
                        ctypes.c_uint64(seed), ctypes.c_uint32(step), ctypes.c_float(G),
                        ctypes.c_float(beta), _p(q), _p(trace), ctypes.c_double(tol),
                        ctypes.byref(st))
    return q, st.as_dict()


def dg_replay_steps(h, J, m, algo, seed, step0, G, beta, q, trace, tol=1e-6):
    """len(G) consecutive dense steps with resident FP64 fields (orc_dg_replay_steps);
    trace holds the steps' words back to back.  Returns (q after the last step, stats)."""
    h, J = _f64(h), _f64(J)
    q = _i8(q).copy()
    G = _f32(np.atleast_1d(G))
    beta = _f32(np.broadcast_to(np.asarray(beta, np.float32), G.shape))
    trace = np.ascontiguousarray(trace, np.uint32).ravel()
    N = len(h)
    words = (N * m + 31) // 32
    if trace.size < words * len(G):
        raise ValueError("trace holds %d words, %d steps need %d" % (trace.size, len(G), words * len(G)))
    st = ReplayStats()
    lib().orc_dg_replay_steps(_p(h), _p(J), ctypes.c_int(N), ctypes.c_int(m), ctypes.c_int(algo),
                              ctypes.c_uint64(seed), ctypes.c_uint32(step0), ctypes.c_int(len(G)),
                              _p(G), _p(beta), _p(q), _p(trace), ctypes.c_double(tol), ctypes.byref(st))
    return q, st.as_dict()


def bg_replay(h0, h1, J, m, algo, seed, step, G, beta, q0, q1, trace, tol=1e-6):
    """One bipartite step in FP64 (h0, h1, J taken as FP64; fp32 inputs convert exactly)."""
    h0, h1, J = _f64(h0), _f64(h1), _f64(J)
    q0, q1 = _i8(q0).copy(), _i8(q1).copy()
    trace = np.ascontiguousarray(trace, np.uint32)
    st = ReplayStats()
    lib().orc_bg_replay(_p(h0), _p(h1), _p(J), ctypes.c_int(len(h0)), ctypes.c_int(len(h1)),
                        ctypes.c_int(m), ctypes.c_int(algo), ctypes.c_uint64(seed),
                        ctypes.c_uint32(step), ctypes.c_float(G), ctypes.c_float(beta),
                        _p(q0), _p(q1), _p(trace), ctypes.c_double(tol), ctypes.byref(st))
    return q0, q1, st.as_dict()
