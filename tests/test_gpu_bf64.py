"""The double-precision brute-force searchers (dtype=numpy.float64) against the
FP64 oracle energies of every state: Emin within 1e-12 relative and the same
argmin set, including a tie that only FP64 breaks."""
import numpy as np
import pytest

import sqaod_gb300 as sq
from oracle import oracle_ctypes as orc

pytestmark = pytest.mark.gpu
F64 = np.float64


def _argmin_set(E, sign, rows):
    s = sign * np.asarray(E, F64)
    best = s.min()
    tol = 1e-12 * max(1., abs(best))
    return best, {rows(i) for i in np.nonzero(s <= best + tol)[0]}


@pytest.mark.parametrize("optimize", ["min", "max"])
def test_dense_bf64_matches_fp64_exhaustive(optimize):
    om, sign = (sq.minimize, 1.) if optimize == "min" else (sq.maximize, -1.)
    rng = np.random.default_rng(21)
    N = 16
    W = rng.uniform(-1, 1, (N, N))
    W = (W + W.T) / 2
    s = sq.cuda.dense_graph_bf_searcher(W, om, dtype=F64)
    s.search()
    E, xs = s.get_E(), s.get_x()
    assert E.dtype == F64 and s.get_preferences()["precision"] == "double"
    X = sq.create_bitset_sequence(range(2 ** N), N)
    best, ref = _argmin_set(orc.dg_energy_qubo(W, X), sign, lambda i: tuple(X[i]))
    assert abs(sign * E[0] - best) <= 1e-12 * max(1., abs(best))
    assert {tuple(x) for x in xs} == ref


def test_dense_bf64_breaks_a_tie_of_fp32():
    # E(1,0,0,0) = -1 and E(0,1,0,0) = -1 - 1e-9: equal in fp32, distinct in FP64
    W = np.zeros((4, 4))
    W[0, 0], W[1, 1] = -1., -1. - 1e-9
    W[0, 1] = W[1, 0] = 2.
    W[2, 2] = W[3, 3] = 0.5
    s64 = sq.cuda.dense_graph_bf_searcher(W, sq.minimize, dtype=F64)
    s64.search()
    assert [x.tolist() for x in s64.get_x()] == [[0, 1, 0, 0]]
    assert s64.get_E()[0] == -1. - 1e-9
    s32 = sq.cuda.dense_graph_bf_searcher(W, sq.minimize, dtype=np.float32)
    s32.search()
    assert sorted(x.tolist() for x in s32.get_x()) == [[0, 1, 0, 0], [1, 0, 0, 0]]


def test_dense_bf64_integer_W_equals_float32():
    rng = np.random.default_rng(22)
    U = rng.integers(-8, 9, (14, 14))
    W = (np.triu(U) + np.triu(U, 1).T).astype(F64)
    a = sq.cuda.dense_graph_bf_searcher(W, sq.minimize, dtype=F64)
    b = sq.cuda.dense_graph_bf_searcher(W.astype(np.float32), sq.minimize)
    a.search()
    b.search()
    assert a.get_E()[0] == b.get_E()[0]
    assert [x.tolist() for x in a.get_x()] == [x.tolist() for x in b.get_x()]


def test_dense_bf64_search_range_equals_search():
    rng = np.random.default_rng(23)
    N = 12
    W = rng.uniform(-1, 1, (N, N))
    W = (W + W.T) / 2
    a = sq.cuda.dense_graph_bf_searcher(W, sq.minimize, dtype=F64, tile_size=512)
    a.prepare()
    while not a.search_range():
        pass
    a.make_solution()
    b = sq.cuda.dense_graph_bf_searcher(W, sq.minimize, dtype=F64)
    b.search()
    assert a.get_E()[0] == b.get_E()[0]
    assert [x.tolist() for x in a.get_x()] == [x.tolist() for x in b.get_x()]


def test_bipartite_bf64_matches_fp64_exhaustive():
    rng = np.random.default_rng(24)
    N0, N1 = 8, 9
    b0, b1 = rng.uniform(-1, 1, N0), rng.uniform(-1, 1, N1)
    W = rng.uniform(-1, 1, (N1, N0))
    s = sq.cuda.bipartite_graph_bf_searcher(b0, b1, W, sq.minimize, dtype=F64)
    s.search()
    E, xs = s.get_E(), s.get_x()
    assert E.dtype == F64 and s.get_preferences()["precision"] == "double"
    X = sq.create_bitset_sequence(range(2 ** (N0 + N1)), N0 + N1)
    x0, x1 = np.ascontiguousarray(X[:, :N0]), np.ascontiguousarray(X[:, N0:])
    best, ref = _argmin_set(orc.bg_energy_qubo(b0, b1, W, x0, x1), 1., lambda i: (tuple(x0[i]), tuple(x1[i])))
    assert abs(E[0] - best) <= 1e-12 * max(1., abs(best))
    assert {(tuple(a), tuple(b)) for a, b in xs} == ref


@pytest.mark.parametrize("bad", [1e39, float("inf")])
def test_bf64_rejects_couplings_beyond_float32(bad):
    """The fp32 screening pass cannot represent such couplings (inf - inf energies
    would drop true minimisers), so the <double> searchers refuse the problem."""
    import sqaod_gb300 as sq
    W = np.zeros((8, 8))
    W[2, 3] = W[3, 2] = bad
    with pytest.raises(RuntimeError, match="float32"):
        sq.cuda.dense_graph_bf_searcher(W, sq.minimize, dtype=F64)
    b0, b1, Wb = np.zeros(4), np.zeros(5), np.zeros((5, 4))
    Wb[1, 1] = bad
    with pytest.raises(RuntimeError, match="float32"):
        sq.cuda.bipartite_graph_bf_searcher(b0, b1, Wb, sq.minimize, dtype=F64)
