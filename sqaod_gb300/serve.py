"""Request server: continuous batching of anneal and search requests of mixed size and type.

Requests (dense or bipartite QUBOs, each with its own trotter count, seed and
G/beta schedule) are admitted in arrival order while their device-memory
footprint fits the budget and a slot is free; one that cannot start yet does
not block the ones behind it.  Every tick() advances every admitted request by
8 annealOneSteps (one field-refresh period); finished requests get their FP64 energies and spins
copied out and free their memory in the same tick.

A request with m > 1 trotters runs SQA with the coloring sweep; m == 1 runs
simulated annealing (sa_naive for dense, sa_coloring for bipartite).  Each
ends in exactly the state the single-instance annealer of
sqaod_gb300.cuda reaches with the same algorithm, seed and schedule (after
prepare() and randomize_spin()).

Dense brute-force searches (N < 64) are served beside the anneals: each tick
searches the next 2^30 states of every active search, and a finished search
gives the exact FP64 minimum and its minimisers, as the single-instance
searcher's search() with the same tile_size does.  No counterpart in the
reference.
"""
import ctypes

import numpy as np

from . import common
from ._lib import call, lib, ptr

QUEUED, ACTIVE, DONE = 0, 1, 2


class AnnealServer:
    def __init__(self, budget_bytes=8 << 30, max_slots=4096):
        self._L = lib()
        h = ctypes.c_void_p()
        call(self._L.sq103_server_new, ctypes.byref(h), ctypes.c_ulonglong(int(budget_bytes)),
             ctypes.c_int(int(max_slots)))
        self._h = h
        self._shape = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.sq103_server_delete(h)
            except Exception:
                pass
            self._h = None

    def _call(self, name, *args):
        return call(getattr(self._L, "sq103_server_" + name), self._h, *args)

    @staticmethod
    def _schedule(G, beta):
        G = np.ascontiguousarray(G, np.float32).ravel()
        beta = np.ascontiguousarray(np.broadcast_to(np.asarray(beta, np.float32), G.shape), np.float32)
        return G, beta

    def submit_dense(self, W, n_trotters, G, beta, optimize=common.minimize, seed=0):
        """Queues a dense QUBO anneal (W symmetric, or triangular as in
        set_qubo); returns its request id."""
        common.check_square(W)
        W = common.fix_type(W, np.float32)
        G, beta = self._schedule(G, beta)
        rid = ctypes.c_int()
        common.submit_symmetric(W, np.float32, lambda w: self._call(
            "submit_dense", ptr(w), ctypes.c_int(w.shape[0]), ctypes.c_int(int(n_trotters)),
            ctypes.c_int(common.optimize_flag(optimize)), ctypes.c_ulonglong(int(seed)), ptr(G), ptr(beta),
            ctypes.c_int(len(G)), ctypes.byref(rid)))
        self._shape[rid.value] = (int(n_trotters), W.shape[0], 0)
        return rid.value

    def submit_bipartite(self, b0, b1, W, n_trotters, G, beta, optimize=common.minimize, seed=0):
        """Queues a bipartite QUBO anneal (W is N1 x N0); returns its request id."""
        b0 = np.ascontiguousarray(b0, np.float32).ravel()
        b1 = np.ascontiguousarray(b1, np.float32).ravel()
        W = np.ascontiguousarray(W, np.float32)
        if W.shape != (len(b1), len(b0)):
            raise ValueError("W must be N1 x N0 (%d x %d), got %s" % (len(b1), len(b0), W.shape))
        G, beta = self._schedule(G, beta)
        rid = ctypes.c_int()
        self._call("submit_bipartite", ptr(b0), ptr(b1), ptr(W), ctypes.c_int(len(b0)), ctypes.c_int(len(b1)),
                   ctypes.c_int(int(n_trotters)), ctypes.c_int(common.optimize_flag(optimize)),
                   ctypes.c_ulonglong(int(seed)), ptr(G), ptr(beta), ctypes.c_int(len(G)), ctypes.byref(rid))
        self._shape[rid.value] = (int(n_trotters), len(b0), len(b1))
        return rid.value

    def submit_search(self, W, optimize=common.minimize, tile_size=1 << 18):
        """Queues a dense brute-force search (W symmetric, or triangular as in
        set_qubo, N < 64); returns its request id.  tile_size caps the number of
        minimisers returned, as the searcher's preference of that name does."""
        common.check_square(W)
        W = common.fix_type(W, np.float32)
        rid = ctypes.c_int()
        common.submit_symmetric(W, np.float32, lambda w: self._call(
            "submit_search", ptr(w), ctypes.c_int(w.shape[0]), ctypes.c_int(common.optimize_flag(optimize)),
            ctypes.c_int(int(tile_size)), ctypes.byref(rid)))
        self._shape[rid.value] = ("search", W.shape[0])
        return rid.value

    def tick(self):
        """8 annealOneSteps of every active request; returns how many finished."""
        c = ctypes.c_int()
        self._call("tick", ctypes.byref(c))
        return c.value

    def state(self, rid):
        s = ctypes.c_int()
        self._call("state", ctypes.c_int(rid), ctypes.byref(s))
        return s.value

    def state_or_none(self, rid):
        """The request's state, or None once it has been released."""
        s = ctypes.c_int()
        if self._L.sq103_server_state(self._h, ctypes.c_int(rid), ctypes.byref(s)) != 0:
            return None
        return s.value

    def inject_status(self, rid, value=1):
        """Fault injection for tests: marks an active dense request as if its
        sweep had given up a bounded device wait.  Its result() then raises;
        every other request is unaffected."""
        self._call("inject_status", ctypes.c_int(rid), ctypes.c_int(int(value)))

    def stats(self):
        v = [ctypes.c_int() for _ in range(3)]
        b = ctypes.c_ulonglong()
        self._call("stats", *[ctypes.byref(x) for x in v], ctypes.byref(b))
        return {"queued": v[0].value, "active": v[1].value, "done": v[2].value, "bytes_in_use": b.value}

    def set_large_limit(self, n):
        """At most n large instances admitted at a time (default 64): dense ones on the
        one-CTA-per-trotter path (packed launches), bipartite ones on the per-instance kernels."""
        self._call("set_large_limit", ctypes.c_int(int(n)))

    def completed(self, cap=4096):
        """Ids of the requests completed since the last call, in completion order."""
        ids = np.zeros(cap, np.int32)
        n = ctypes.c_int()
        self._call("completed", ptr(ids), ctypes.c_int(cap), ctypes.byref(n))
        return ids[:n.value].tolist()

    def result(self, rid, release=True):
        """(E, q) of a finished anneal: m FP64 energies and the spins, q of
        shape (m, N) for dense or a pair ((m, N0), (m, N1)) for bipartite.
        (E, x) of a finished search: the FP64 minimum and its minimisers, x of
        shape (n, N) with bits 0/1."""
        if self._shape[rid][0] == "search":
            return self._search_result(rid, release)
        m, N0, N1 = self._shape[rid]
        E = np.zeros(m, np.float64)
        q0 = np.zeros((m, N0), np.int8)
        q1 = np.zeros((m, max(N1, 1)), np.int8)
        mm = ctypes.c_int()
        cap = max(q0.nbytes, q1.nbytes)
        try:
            self._call("result", ctypes.c_int(rid), ptr(E), ctypes.c_int(m), ctypes.byref(mm), ptr(q0), ptr(q1),
                       ctypes.c_longlong(cap), ctypes.c_int(1 if release else 0))
        finally:
            # a request whose sweep gave up a device wait raises here, and is released all the same
            if release and self.state_or_none(rid) is None:
                self._shape.pop(rid, None)
        if N1 == 0:
            return E, q0
        return E, (q0, q1[:, :N1])

    def _search_result(self, rid, release):
        N = self._shape[rid][1]
        rows = ctypes.c_int()
        self._call("result_rows", ctypes.c_int(rid), ctypes.byref(rows))
        n = rows.value
        E = np.zeros(1, np.float64)
        x = np.zeros((max(n, 1), N), np.int8)
        got = ctypes.c_int()
        self._call("result", ctypes.c_int(rid), ptr(E), ctypes.c_int(1), ctypes.byref(got), ptr(x), ptr(x),
                   ctypes.c_longlong(x.nbytes), ctypes.c_int(1 if release else 0))
        if release:
            self._shape.pop(rid, None)
        return float(E[0]), x[:n]

    def run(self, max_ticks=None):
        """Ticks until nothing is queued or active; returns the number of ticks."""
        n = 0
        while True:
            s = self.stats()
            if s["queued"] == 0 and s["active"] == 0:
                return n
            if max_ticks is not None and n >= max_ticks:
                return n
            self.tick()
            n += 1
