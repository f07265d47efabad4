"""wildqat adapter: wildqat's `opt` class with its `sa()` and `sqa()` run by
this package's CUDA dense annealer (sqaodpy/sqaod/wildqat/opt.py:5-67).

    from sqaod_gb300.wildqat import opt
    a = opt()
    a.qubo = W
    x = a.sa()

It needs the wildqat package (a subclass of `wildqat.opt`); the schedule
attributes it reads (Ts, Tf, R, ite for SA; Gs, Gf, tro for SQA) and `qi()`
are wildqat's.  The annealing loops follow the reference adapter: SA runs
sa_naive with one trotter, ceil(ite / N) sweeps at every temperature, and
records the energy after each; SQA runs the default algorithm with `tro`
trotters, ceil(ite / (N tro)) sweeps at every G with beta = 1 / Tf, and
records the system energy at the end of each G.
"""
import numpy as np

try:
    import wildqat as _wildqat
except ImportError as e:  # pragma: no cover - depends on the environment
    raise ImportError("sqaod_gb300.wildqat needs the wildqat package: %s" % e)

from . import common


class opt(_wildqat.opt):

    def __init__(self, pkg=None, dtype=np.float32):
        _wildqat.opt.__init__(self)
        if pkg is None:
            from . import cuda as pkg
        self.ann = pkg.dense_graph_annealer(dtype=dtype)

    def sa(self):
        """Simulated annealing of `qubo`; returns the bits of the solution."""
        self.E = []
        if len(self.qubo) != 0:
            self.ann.set_qubo(np.array(self.qubo), common.minimize)
            self.ann.set_preferences(algorithm=common.algorithm.sa_naive, n_trotters=1)
        self.ann.prepare()
        self.ann.randomize_spin()
        N = self.ann.get_problem_size()
        sweeps = -(-self.ite // N)
        T = self.Ts
        while T > self.Tf:
            for _ in range(sweeps):
                self.ann.anneal_one_step(T, 1.)
                self.E.append(self.ann.get_system_E(0., 0.))  # SA ignores G and beta here
            T *= self.R
        return self.ann.get_x()[0]

    def sqa(self):
        """Simulated quantum annealing of `qubo`; returns the bits of every trotter."""
        self.E = []
        if len(self.qubo) != 0:
            self.ann.set_qubo(np.array(self.qubo), common.minimize)
            self.ann.set_preferences(algorithm=common.algorithm.default, n_trotters=self.tro)
            self.qi()
        self.ann.prepare()
        self.ann.randomize_spin()
        N = self.ann.get_problem_size()
        sweeps = -(-self.ite // (N * self.tro))
        beta = 1. / self.Tf
        G = self.Gs
        while G > self.Gf:
            for _ in range(sweeps):
                self.ann.anneal_one_step(G, beta)
            self.E.append(self.ann.get_system_E(G, beta))
            G *= self.R
        return self.ann.get_x()
