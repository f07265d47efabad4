"""The wildqat adapter on the GPU, with a stand-in for the wildqat package
(not installed here): its opt base class only carries the schedule
attributes the adapter reads, with values chosen for this test."""
import importlib
import sys
import types

import numpy as np
import pytest

import sqaod_gb300 as sq

pytestmark = pytest.mark.gpu


def stand_in():
    mod = types.ModuleType("wildqat")

    class opt:
        def __init__(self):
            self.Ts, self.Tf, self.R, self.ite = 5., 0.02, 0.9, 600
            self.Gs, self.Gf, self.tro = 5., 0.02, 8
            self.qubo = []
            self.qi_calls = 0

        def qi(self):
            self.qi_calls += 1

    mod.opt = opt
    return mod


@pytest.fixture
def wq(monkeypatch):
    monkeypatch.setitem(sys.modules, "wildqat", stand_in())
    monkeypatch.delitem(sys.modules, "sqaod_gb300.wildqat", raising=False)
    return importlib.import_module("sqaod_gb300.wildqat")


def exact_min(W):
    s = sq.cuda.dense_graph_bf_searcher(W, sq.minimize)
    s.search()
    return float(s.get_E()[0])


def test_wildqat_sa_and_sqa_reach_the_exact_minimum(wq):
    rng = np.random.default_rng(0)
    N = 12
    W = rng.uniform(-1, 1, (N, N))
    W = ((W + W.T) / 2).astype(np.float32)
    Emin = exact_min(W)

    a = wq.opt()
    a.qubo = W
    a.ann.seed(1)
    x = np.asarray(a.sa())
    assert x.shape == (N,)
    assert np.isclose(float(x @ W.astype(np.float64) @ x), Emin, atol=1e-5)
    n_T = int(np.ceil(np.log(a.Tf / a.Ts) / np.log(a.R)))
    assert len(a.E) == n_T * -(-a.ite // N)

    b = wq.opt()
    b.qubo = W
    b.ann.seed(2)
    xs = [np.asarray(v) for v in b.sqa()]
    assert len(xs) == b.tro and b.qi_calls == 1
    assert np.isclose(min(float(v @ W.astype(np.float64) @ v) for v in xs), Emin, atol=1e-5)
