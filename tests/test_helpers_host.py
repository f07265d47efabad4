"""Python helpers above the solver API that need no GPU: make_summary and
unique_x (sqaodpy/sqaod/common/summary.py)."""
import numpy as np
import pytest

import sqaod_gb300 as sq


class FakeSolver:
    def __init__(self, E, xs, opt):
        self._E, self._xs, self._opt = np.asarray(E, np.float32), xs, opt

    def get_E(self):
        return self._E

    def get_x(self):
        return self._xs

    def get_optimize_dir(self):
        return self._opt


def bits(s):
    return np.array([int(c) for c in s], np.int8)


def test_make_summary_keeps_distinct_best_solutions_in_bit_order():
    xs = [bits("110"), bits("011"), bits("110"), bits("000"), bits("010")]
    s = sq.make_summary(FakeSolver([-2., -2., -2., 1., -1.], xs, sq.minimize))
    assert s.E == -2.
    assert [x.tolist() for x in s.xlist] == [[0, 1, 1], [1, 1, 0]]
    s = sq.make_summary(FakeSolver([-2., -2., -2., 1., -1.], xs, sq.maximize))
    assert s.E == 1. and [x.tolist() for x in s.xlist] == [[0, 0, 0]]
    assert sq.make_summary().__class__ is sq.Summary


def test_unique_x_of_bipartite_pairs_orders_by_x1_first():
    pairs = [(bits("10"), bits("01")), (bits("01"), bits("10")), (bits("00"), bits("01")), (bits("10"), bits("01"))]
    u = sq.unique_x(pairs)
    assert [(a.tolist(), b.tolist()) for a, b in u] == [([0, 0], [0, 1]), ([1, 0], [0, 1]), ([0, 1], [1, 0])]


def test_batch_routing_threshold_rules():
    # host-side rules of the batch's routing threshold (no device work before prepare)
    from sqaod_gb300.batch import DenseBatchAnnealer
    b = DenseBatchAnnealer()
    with pytest.raises(sq.SqaodError, match="must not be negative"):
        b.set_multicta_min_n(-1)
    b.set_multicta_min_n(0)
    assert b.multicta_count() == 0


def test_checkpoint_needs_a_prepared_annealer():
    a = sq.cuda.dense_graph_annealer()
    state = {"q": np.ones((2, 4), np.int8), "F": np.zeros((2, 4), np.float32), "seed": 1, "step": 0,
             "since_refresh": 0}
    with pytest.raises(sq.SqaodError, match="not set"):
        a.set_checkpoint(state)
    with pytest.raises(RuntimeError, match="same shape"):
        a.set_checkpoint(dict(state, F=np.zeros((3, 4), np.float32)))
