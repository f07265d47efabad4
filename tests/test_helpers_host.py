"""Python helpers above the solver API that need no GPU: make_summary and
unique_x (sqaodpy/sqaod/common/summary.py)."""
import numpy as np

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
