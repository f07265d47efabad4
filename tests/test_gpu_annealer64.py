"""The <double> annealers (dtype numpy.float64; sqaod::cuda::{Dense,Bipartite}
GraphAnnealer<double>) through the C ABI.

Their sweeps run on the fp32 rounding of the FP64 couplings and decide every
flagged trial from the FP64 couplings, so they replay against the FP64 host
replay of the FP64 problem itself: a decision may differ only where the FP64
acceptance margin is below 1e-6 (counted).  The couplings below are not
representable in fp32, so replaying with their fp32 rounding would not do.
Energies and the Hamiltonian are FP64 (1e-12 relative of the oracle).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MARGIN_TOL = 1e-6


@pytest.fixture(scope="module")
def sq():
    import sqaod_gb300
    return sqaod_gb300


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b))) / max(1.0, float(np.max(np.abs(b))))


def _sym64(rng, N):
    W = rng.uniform(-1, 1, (N, N)) + 1e-9 * rng.standard_normal((N, N))
    return np.triu(W) + np.triu(W, 1).T


@pytest.mark.parametrize("N,m,algo,opt", [(96, 8, "coloring", "min"), (130, 5, "coloring", "max"),
                                          (1100, 16, "coloring", "min"), (64, 6, "sa_naive", "min"),
                                          (48, 4, "coloring", "max")])
def test_dense_annealer64_replays_fp64(sq, orc, N, m, algo, opt):
    rng = np.random.default_rng(N + m)
    W = _sym64(rng, N)
    assert not np.array_equal(W.astype(np.float32).astype(np.float64), W)
    om = sq.maximize if opt == "max" else sq.minimize
    a = sq.cuda.dense_graph_annealer(W, om, dtype=np.float64, n_trotters=m, algorithm=algo)
    assert a.get_preferences()["precision"] == "double"
    h, J, c = a.get_hamiltonian()
    assert h.dtype == np.float64 and J.dtype == np.float64
    h0, J0, c0 = orc.dg_hamiltonian(-W if opt == "max" else W)
    assert _rel(h, h0) <= 1e-14 and _rel(J, J0) <= 1e-14 and abs(c - c0) <= 1e-12 * max(1.0, abs(c0))
    a.seed(17)
    a.prepare()
    a.randomize_spin()
    q = np.array(a.get_q())
    a.set_trace(True)
    _, step0 = a.get_rng_state()
    G = np.array([4.0, 2.0, 1.0, 0.5, 0.2, 0.1, 0.05, 0.03, 0.02, 0.01], np.float32)
    a.anneal(G, 30.0)
    trace = a.get_trace((N * m + 31) // 32 * len(G))
    code = {"coloring": orc.ALGO_COLORING, "sa_naive": orc.ALGO_SA_NAIVE, "naive": orc.ALGO_NAIVE}[algo]
    q_host, st = orc.dg_replay_steps(h, J, m, code, 17, step0, G, 30.0, q, trace, MARGIN_TOL)
    print("N=%d m=%d %s %s: %s" % (N, m, algo, opt, st))
    qd = np.array(a.get_q())
    assert np.array_equal(qd, q_host)
    assert st["n_mismatch"] == st["n_mismatch_small"], st
    a.make_solution()
    E = a.get_E()
    assert E.dtype == np.float64
    E_ref = orc.dg_energy_ising(h0, J0, c0, qd) * (-1 if opt == "max" else 1)
    assert _rel(E, E_ref) <= 1e-12


@pytest.mark.parametrize("N0,N1,m,algo", [(40, 24, 6, "coloring"), (1024, 1024, 8, "coloring"),
                                          (33, 17, 5, "sa_coloring")])
def test_bipartite_annealer64_replays_fp64(sq, orc, N0, N1, m, algo):
    rng = np.random.default_rng(N0 + N1 + m)
    b0 = rng.uniform(-1, 1, N0) + 1e-9
    b1 = rng.uniform(-1, 1, N1) - 1e-9
    W = rng.uniform(-1, 1, (N1, N0)) + 1e-9 * rng.standard_normal((N1, N0))
    a = sq.cuda.bipartite_graph_annealer(b0, b1, W, dtype=np.float64, n_trotters=m, algorithm=algo)
    assert a.get_preferences()["precision"] == "double"
    h0, h1, J, c = a.get_hamiltonian()
    r0, r1, rJ, rc = orc.bg_hamiltonian(b0, b1, W)
    assert _rel(h0, r0) <= 1e-14 and _rel(h1, r1) <= 1e-14 and _rel(J, rJ) <= 1e-14
    a.seed(5)
    a.prepare()
    a.randomize_spin()
    pairs = a.get_q()
    q0 = np.array([p[0] for p in pairs])
    q1 = np.array([p[1] for p in pairs])
    a.set_trace(True)
    code = {"coloring": orc.ALGO_COLORING, "sa_coloring": orc.ALGO_SA_COLORING}[algo]
    tot = {}
    for G in (3.0, 1.0, 0.3, 0.05):
        _, step = a.get_rng_state()
        a.anneal_one_step(G, 20.0)
        trace = a.get_trace((m * (N0 + N1) + 31) // 32)
        q0, q1, st = orc.bg_replay(h0, h1, J, m, code, 5, step, G, 20.0, q0, q1, trace, MARGIN_TOL)
        pairs = a.get_q()
        assert np.array_equal(np.array([p[0] for p in pairs]), q0)
        assert np.array_equal(np.array([p[1] for p in pairs]), q1)
        for k, v in st.items():
            tot[k] = max(tot.get(k, 0), v) if k == "max_mismatch_margin" else tot.get(k, 0) + v
    print("bipartite N0=%d N1=%d m=%d %s: %s" % (N0, N1, m, algo, tot))
    assert tot["n_mismatch"] == tot["n_mismatch_small"], tot
    a.make_solution()
    E = a.get_E()
    assert E.dtype == np.float64
    assert _rel(E, orc.bg_energy_ising(r0, r1, rJ, rc, q0, q1)) <= 1e-12


def test_annealer64_known_answers_and_system_E(sq):
    """W = +-ones reach E = 0 (sqaodpy/tests/test_dense_graph_annealer.py:202-262)
    in float64, and getSystemE follows the reference's identity."""
    N, m = 16, 4
    for sign in (1.0, -1.0):
        a = sq.cuda.dense_graph_annealer(sign * np.ones((N, N)), dtype=np.float64, n_trotters=m)
        a.seed(1)
        a.prepare()
        a.randomize_spin()
        G = 5.0
        while G > 0.01:
            a.anneal_one_step(G, 50.0)
            G *= 0.95
        a.make_solution()
        E = a.get_E()
        assert abs(E.min() - (0.0 if sign > 0 else -N * N)) < 1e-9
        sysE = a.get_system_E(0.5, 50.0)
        assert isinstance(sysE, np.float64)
