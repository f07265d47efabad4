"""Batched dense annealing: many independent QUBO instances in lock-step.

Every annealOneStep of all instances is one persistent kernel launch,
replayed from a CUDA graph, with instances taken from a queue largest first.
Each instance follows exactly the rules of the single-instance annealer
(coloring sweep, sa_naive for one trotter, Philox stream of its seed, field refresh every 8 steps), so
an instance annealed in a batch ends in the same state as when annealed alone
with sqaod_gb300.cuda.dense_graph_annealer and the same seed.
"""
import ctypes

import numpy as np

from . import common
from ._lib import call, lib, ptr


class DenseBatchAnnealer:
    def __init__(self):
        self._L = lib()
        h = ctypes.c_void_p()
        call(self._L.sq103_dense_batch_new, ctypes.byref(h))
        self._h = h
        self._m = []
        self._N = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.sq103_dense_batch_delete(h)
            except Exception:
                pass
            self._h = None

    def _call(self, name, *args):
        return call(getattr(self._L, "sq103_dense_batch_" + name), self._h, *args)

    def add(self, W, n_trotters, optimize=common.minimize, seed=0):
        """Adds one QUBO instance; returns its index."""
        common.check_square(W)
        W = common.fix_type(W, np.float32)
        idx = ctypes.c_int()
        common.submit_symmetric(W, np.float32, lambda w: self._call(
            "add", ptr(w), ctypes.c_int(w.shape[0]), ctypes.c_int(int(n_trotters)),
            ctypes.c_int(common.optimize_flag(optimize)), ctypes.c_ulonglong(int(seed)), ctypes.byref(idx)))
        self._m.append(int(n_trotters))
        self._N.append(W.shape[0])
        return idx.value

    def set_schedule(self, G, beta):
        G = np.ascontiguousarray(G, np.float32)
        beta = np.ascontiguousarray(np.broadcast_to(np.asarray(beta, np.float32), G.shape), np.float32)
        self._call("set_schedule", ptr(G), ptr(beta), ctypes.c_int(len(G)))

    def prepare(self):
        self._call("prepare")

    def set_multicta_min_n(self, N):
        """Instances of at least N spins run on the one-CTA-per-trotter sweep
        (packed launches); 0 keeps all on the persistent kernel.  Default 1024;
        results do not depend on it.  Takes effect at the next prepare()."""
        self._call("set_multicta_min_n", ctypes.c_int(N))

    def multicta_count(self):
        n = ctypes.c_int()
        self._call("multicta_count", ctypes.byref(n))
        return n.value

    def autotune_routing(self, trial_steps=8, candidates=(0, 512, 768, 1024, 1400, 2048)):
        """Chooses, by timing trial_steps steps from the start of the schedule,
        the size limit at and above which instances take one CTA per trotter
        (set_multicta_min_n); prepares the batch again with it and returns it.
        The results do not depend on the choice."""
        c = np.ascontiguousarray(candidates, np.int32)
        chosen = ctypes.c_int()
        self._call("autotune_routing", ctypes.c_int(int(trial_steps)), ptr(c), ctypes.c_int(len(c)),
                   ctypes.byref(chosen))
        return chosen.value

    def autotune(self, trial_steps=2):
        s = ctypes.c_int()
        self._call("autotune", ctypes.c_int(trial_steps), ctypes.byref(s))
        return s.value

    def anneal(self, n_steps, use_graph=True):
        self._call("anneal", ctypes.c_int(n_steps), ctypes.c_int(1 if use_graph else 0))

    def sync(self):
        self._call("sync")

    def info(self):
        v = [ctypes.c_int() for _ in range(4)]
        self._call("info", *[ctypes.byref(x) for x in v])
        return {"instances": v[0].value, "position": v[1].value, "grid": v[2].value, "smem_bytes": v[3].value}

    def get_E64(self, index):
        m = self._m[index]
        E = np.zeros(m, np.float64)
        n = ctypes.c_int()
        self._call("get_E", ctypes.c_int(index), ptr(E), ctypes.c_int(m), ctypes.byref(n))
        return E

    def get_q(self, index):
        m, N = self._m[index], self._N[index]
        q = np.zeros((m, N), np.int8)
        n = ctypes.c_int()
        self._call("get_q", ctypes.c_int(index), ptr(q), ctypes.c_int(m), ctypes.byref(n))
        return q
