"""GPU parity tests: the CUDA path (through the C ABI) against the CPU oracle.

- QUBO -> Ising (h, J, c) and FP64 energies within 1e-5 relative of the FP64
  oracle and of the reference numpy golden vectors;
- every annealer sweep replays against the FP64 host replay of the same
  Philox stream: each decision must agree unless its acceptance margin
  |min(1, exp(-rate dE)) - u| is below 1e-6 (those are counted);
- brute-force Emin and argmin sets bit-exact with the reference CPU searcher
  on integer-valued W;
- the reference tests' known answers (sqaodpy/tests/test_dense_graph_annealer.py,
  test_bipartite_graph_annealer.py, test_dense_graph_bf_searcher.py).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5      # formulas / energies vs FP64
MARGIN_TOL = 1e-6   # replay: decisions may differ only below this acceptance margin


@pytest.fixture(scope="module")
def sq():
    import sqaod_gb300
    return sqaod_gb300


def rand_sym(rng, N, lo=-1., hi=1.):
    W = rng.uniform(lo, hi, (N, N))
    W = np.triu(W) + np.triu(W, 1).T
    return W.astype(np.float32)


def bits_to_int(bits):
    v = 0
    for b in bits:
        v = (v << 1) | int(b)
    return v


def rel_close(a, b, tol=REL_TOL):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(1.0, float(np.max(np.abs(b))) if b.size else 1.0)
    return float(np.max(np.abs(a - b))) <= tol * scale if b.size else True


# ------------------------------------------------------------- formulas
@pytest.mark.parametrize("om", [0, 1])
def test_dense_hamiltonian_vs_fp64(sq, orc, om):
    rng = np.random.default_rng(11)
    W = rand_sym(rng, 100)
    a = sq.cuda.dense_graph_annealer(W, sq.maximize if om else sq.minimize)
    h, J, c = a.get_hamiltonian()
    h0, J0, c0 = orc.dg_hamiltonian(-W.astype(np.float64) if om else W)
    assert rel_close(h, h0) and rel_close(J, J0) and rel_close([c], [c0])


def test_dense_hamiltonian_golden(sq, golden):
    for name in ("ex8", "r16", "r100"):
        a = sq.cuda.dense_graph_annealer(golden["dg_%s_W" % name].astype(np.float32))
        h, J, c = a.get_hamiltonian()
        assert rel_close(h, golden["dg_%s_h" % name]) and rel_close(J, golden["dg_%s_J" % name])
        assert rel_close([c], [golden["dg_%s_c" % name]])


def test_dense_set_qubo_triangular_input(sq):
    """A triangular W is accepted as (W + W^T) / 2 (the native check sees the
    asymmetric W first and the host then symmetrizes it), for the annealer and
    the brute-force searcher alike."""
    rng = np.random.default_rng(5)
    for make, N in ((sq.cuda.dense_graph_annealer, 40), (sq.cuda.dense_graph_bf_searcher, 16)):
        S = rand_sym(rng, N)
        U = np.triu(S) * 2 - np.diag(np.diag(S))
        for T in (U, U.T.copy()):  # upper and lower triangles (sqaodpy/tests/test_symmetrize_solvers.py)
            a, b = make(T), make(S)
            if hasattr(a, "get_hamiltonian"):
                for x, y in zip(a.get_hamiltonian(), b.get_hamiltonian()):
                    assert rel_close(x, y, 1e-6)
            else:
                a.search()
                b.search()
                assert rel_close(a.get_E(), b.get_E(), 1e-6)


def test_dense_set_qubo_rejects_asymmetric(sq):
    """The exact symmetry check runs on the device copy, before any state
    changes: an asymmetric W is rejected and the previous problem stays."""
    rng = np.random.default_rng(9)
    S = rand_sym(rng, 70)
    a = sq.cuda.dense_graph_annealer(S)
    h0, J0, c0 = a.get_hamiltonian()
    for r, c in ((3, 60), (69, 0), (33, 32)):  # inside, corner and diagonal-adjacent tiles
        B = S.copy()
        B[r, c] += 0.5
        with pytest.raises(RuntimeError, match="symmetric"):
            a.set_qubo(B)
        h1, J1, c1 = a.get_hamiltonian()
        assert np.array_equal(h0, h1) and np.array_equal(J0, J1) and c0 == c1


def test_dense_energy_all_states_golden(sq, golden):
    W, X = golden["dg_r8_W"].astype(np.float32), golden["dg_r8_X"]
    a = sq.cuda.dense_graph_annealer(W)
    a.set_qset([sq.bit_to_spin(x).astype(np.int8) for x in X])
    assert rel_close(a.get_E(), golden["dg_r8_E"])
    assert rel_close(a.get_E64(), golden["dg_r8_E"])


def test_dense_energy_vs_fp64_large(sq, orc):
    rng = np.random.default_rng(5)
    N, m = 300, 12
    W = rand_sym(rng, N)
    a = sq.cuda.dense_graph_annealer(W, n_trotters=m)
    a.seed(1)
    a.prepare()
    a.randomize_spin()
    q = np.array(a.get_q())
    h, J, c = orc.dg_hamiltonian(W)
    # the precision criterion: within 1e-5 relative of the all-FP64 oracle
    assert rel_close(a.get_E(), orc.dg_energy_ising(h, J, c, q))
    # the FP64 evaluation itself: exact up to rounding, given the fp32 h and J the API stores
    h32, J32, _ = a.get_hamiltonian()
    assert rel_close(a.get_E64(), orc.dg_energy_ising(h32, J32, c, q), 1e-11)


def test_known_energies(sq):
    N = 8
    a = sq.cuda.dense_graph_annealer(np.ones((N, N), np.float32), n_trotters=1)
    a.prepare()
    a.set_q(np.ones(N, np.int8))
    E = a.get_E()
    assert len(E) == 1 and E[0] == N * N
    assert np.all(a.get_x()[0] == 1)
    a.set_q(-np.ones(N, np.int8))
    assert abs(a.get_E()[0]) < 1e-6
    b = sq.cuda.bipartite_graph_annealer(np.ones(4, np.float32), np.ones(4, np.float32),
                                         np.ones((4, 4), np.float32), n_trotters=1)
    b.prepare()
    b.set_q((np.ones(4, np.int8), np.ones(4, np.int8)))
    assert b.get_E()[0] == 4 * 4 + 4 + 4


def test_get_x_is_the_bits_of_the_spins(sq):
    """x = (q + 1) / 2 on every target: char is unsigned on aarch64, where a
    spin read as plain char would turn -1 into 255."""
    rng = np.random.default_rng(0)
    a = sq.cuda.dense_graph_annealer(rand_sym(rng, 12), sq.minimize, n_trotters=3)
    a.seed(1)
    a.prepare()
    a.randomize_spin()
    for q, x in zip(a.get_q(), a.get_x()):
        assert set(np.unique(q)) <= {-1, 1} and np.array_equal(x, (q + 1) // 2)
    b = sq.cuda.bipartite_graph_annealer(rng.uniform(-1, 1, 5).astype(np.float32),
                                         rng.uniform(-1, 1, 7).astype(np.float32),
                                         rng.uniform(-1, 1, (7, 5)).astype(np.float32), n_trotters=2)
    b.seed(2)
    b.prepare()
    b.randomize_spin()
    for (q0, q1), (x0, x1) in zip(b.get_q(), b.get_x()):
        assert np.array_equal(x0, (q0 + 1) // 2) and np.array_equal(x1, (q1 + 1) // 2)


def test_bipartite_formulas_golden(sq, golden):
    g = golden
    b = sq.cuda.bipartite_graph_annealer(g["bg_b0"], g["bg_b1"], g["bg_W"])
    h0, h1, J, c = b.get_hamiltonian()
    assert rel_close(h0, g["bg_h0"]) and rel_close(h1, g["bg_h1"]) and rel_close(J, g["bg_J"])
    assert rel_close([c], [g["bg_c"]])
    q0 = (2 * g["bg_x0"] - 1).astype(np.int8)
    q1 = (2 * g["bg_x1"] - 1).astype(np.int8)
    b.set_qset(list(zip(q0, q1)))
    assert rel_close(b.get_E(), g["bg_E"])


def test_bipartite_hamiltonian_vs_fp64_maximize(sq, orc):
    rng = np.random.default_rng(3)
    N0, N1 = 70, 45
    b0, b1 = rng.uniform(-1, 1, N0).astype(np.float32), rng.uniform(-1, 1, N1).astype(np.float32)
    W = rng.uniform(-1, 1, (N1, N0)).astype(np.float32)
    b = sq.cuda.bipartite_graph_annealer(b0, b1, W, sq.maximize)
    h0, h1, J, c = b.get_hamiltonian()
    r = orc.bg_hamiltonian(-b0.astype(np.float64), -b1.astype(np.float64), -W.astype(np.float64))
    assert rel_close(h0, r[0]) and rel_close(h1, r[1]) and rel_close(J, r[2]) and rel_close([c], [r[3]])


# ---------------------------------------------------------- sweep replay
DENSE_ALGOS = {"coloring": 1, "naive": 0, "sa_naive": 2}


@pytest.mark.parametrize("algo", ["coloring", "sa_naive"])
@pytest.mark.parametrize("N,m", [(48, 8), (37, 7), (64, 2)])
def test_dense_sweep_replays_fp64(sq, orc, algo, N, m):
    rng = np.random.default_rng(N * 100 + m)
    W = rand_sym(rng, N)
    a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm=algo)
    seed = 1234 + N
    a.seed(seed)
    a.prepare()
    a.randomize_spin()
    q = np.array(a.get_q())
    assert np.array_equal(q, orc.gpu_randomize(seed, 0, 0, m, N))
    h, J, c = a.get_hamiltonian()
    a.set_trace(True)
    nwords = (N * m + 31) // 32
    schedule = [(3.0, 10.0), (1.0, 10.0), (0.3, 20.0), (0.05, 50.0)]
    for G, beta in schedule:
        _, step = a.get_rng_state()
        a.anneal_one_step(G, beta)
        trace = a.get_trace(nwords)
        q_host, st = orc.dg_replay(h, J, m, DENSE_ALGOS[algo], seed, step, G, beta, q, trace, MARGIN_TOL)
        q = np.array(a.get_q())
        assert np.array_equal(q, q_host), "device state diverged from the replayed trace"
        assert st["n_trials"] == N * m
        assert st["n_mismatch"] == st["n_mismatch_small"], st


BIP_ALGOS = {"naive": 0, "coloring": 1, "sa_naive": 2, "sa_coloring": 3}


@pytest.mark.parametrize("algo", ["coloring", "sa_coloring"])
@pytest.mark.parametrize("N0,N1,m", [(40, 24, 6), (17, 33, 5)])
def test_bipartite_sweep_replays_fp64(sq, orc, algo, N0, N1, m):
    rng = np.random.default_rng(N0 * 7 + N1 + m)
    b0, b1 = rng.uniform(-1, 1, N0).astype(np.float32), rng.uniform(-1, 1, N1).astype(np.float32)
    W = rng.uniform(-1, 1, (N1, N0)).astype(np.float32)
    a = sq.cuda.bipartite_graph_annealer(b0, b1, W, n_trotters=m, algorithm=algo)
    seed = 99 + m
    a.seed(seed)
    a.prepare()
    a.randomize_spin()
    pairs = a.get_q()
    q0 = np.array([p[0] for p in pairs])
    q1 = np.array([p[1] for p in pairs])
    assert np.array_equal(q0, orc.gpu_randomize(seed, 0, 0, m, N0))
    assert np.array_equal(q1, orc.gpu_randomize(seed, 0, 1, m, N1))
    h0, h1, J, c = a.get_hamiltonian()
    a.set_trace(True)
    nbits = m * (N0 + N1) * (m if algo == "sa_naive" else 1)
    for G, beta in [(3.0, 10.0), (0.5, 20.0), (0.05, 50.0)]:
        _, step = a.get_rng_state()
        a.anneal_one_step(G, beta)
        trace = a.get_trace((nbits + 31) // 32)
        r0, r1, st = orc.bg_replay(h0, h1, J, m, BIP_ALGOS[algo], seed, step, G, beta, q0, q1, trace,
                                   MARGIN_TOL)
        pairs = a.get_q()
        q0 = np.array([p[0] for p in pairs])
        q1 = np.array([p[1] for p in pairs])
        assert np.array_equal(q0, r0) and np.array_equal(q1, r1)
        assert st["n_mismatch"] == st["n_mismatch_small"], st


@pytest.mark.parametrize("algo", ["coloring", "sa_naive"])
@pytest.mark.parametrize("N,m", [(128, 16), (256, 7), (96, 2), (512, 64), (130, 16), (1023, 37)])
def test_dense_multi_cta_equals_single_cta(sq, algo, N, m):
    """One CTA per trotter (cooperative) and one CTA per instance run the same
    trials with the same fp32 arithmetic: spins and FP64 energies bit-identical."""
    rng = np.random.default_rng(N + m)
    W = rand_sym(rng, N)
    G = [5.0 * 0.9 ** k for k in range(12)]
    out = []
    for flags in (1, 2):
        a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm=algo)
        a.set_kernel(flags)
        a.seed(21)
        a.prepare()
        a.randomize_spin()
        a.anneal(np.array(G, np.float32), 20.0)
        out.append((np.array(a.get_q()), a.get_E64(), a.get_accepted()))
    assert out[0][2] == out[1][2]
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("N,m", [(4096, 256), (2048, 131)])
def test_dense_multi_cta_equals_single_cta_large(sq, N, m):
    """The benchmark shape (and an odd trotter count): trotters drift apart far
    more at large N, so the neighbour synchronisation is exercised beyond the
    lock-step regime of the small shapes.  Bit-identical to one CTA."""
    rng = np.random.default_rng(N + m)
    W = rand_sym(rng, N)
    G = np.array([5.0, 0.9, 0.2, 0.05], np.float32)
    out = []
    for flags in (1, 2):
        a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm="coloring")
        a.set_kernel(flags)
        a.seed(3)
        a.prepare()
        a.randomize_spin()
        a.anneal(G, 50.0)
        out.append((np.array(a.get_q()), a.get_E64(), a.get_accepted()))
    assert out[0][2] == out[1][2]
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("flags", [1, 2])
@pytest.mark.parametrize("algo,N,m", [("sa_naive", 1023, 8), ("coloring", 1023, 37), ("coloring", 97, 5)])
def test_dense_multi_step_launch_replays_fp64(sq, orc, flags, algo, N, m):
    """Several steps in one launch (anneal over a schedule), odd N and odd
    phase counts per step, both kernels: every step replays against FP64."""
    rng = np.random.default_rng(N + m)
    W = rand_sym(rng, N)
    G = np.array([5.0 * 0.9 ** k for k in range(3)], np.float32)
    a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm=algo)
    a.set_kernel(flags)
    a.seed(21)
    a.prepare()
    a.randomize_spin()
    q = np.array(a.get_q())
    h, J, c = a.get_hamiltonian()
    a.set_trace(True)
    _, step0 = a.get_rng_state()
    a.anneal(G, 20.0)
    nw = (N * m + 31) // 32
    trace = np.array(a.get_trace(nw * len(G)), np.uint32).reshape(len(G), nw)
    for s in range(len(G)):
        q, st = orc.dg_replay(h, J, m, DENSE_ALGOS[algo], 21, step0 + s, float(G[s]), 20.0, q, trace[s], MARGIN_TOL)
        assert st["n_mismatch"] == st["n_mismatch_small"], (s, st)
    assert np.array_equal(np.array(a.get_q()), q)


@pytest.mark.parametrize("algo", ["coloring", "sa_naive"])
def test_dense_multi_cta_replays_fp64(sq, orc, algo):
    N, m = 160, 9
    rng = np.random.default_rng(77)
    W = rand_sym(rng, N)
    a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm=algo)
    a.set_kernel(2)
    a.seed(5)
    a.prepare()
    a.randomize_spin()
    q = np.array(a.get_q())
    h, J, c = a.get_hamiltonian()
    a.set_trace(True)
    for G, beta in [(2.0, 10.0), (0.2, 30.0), (0.02, 50.0)]:
        _, step = a.get_rng_state()
        a.anneal_one_step(G, beta)
        trace = a.get_trace((N * m + 31) // 32)
        q_host, st = orc.dg_replay(h, J, m, DENSE_ALGOS[algo], 5, step, G, beta, q, trace, MARGIN_TOL)
        q = np.array(a.get_q())
        assert np.array_equal(q, q_host)
        assert st["n_mismatch"] == st["n_mismatch_small"], st


def test_dense_anneal_schedule_equals_steps(sq):
    """anneal(G[], beta[]) in one call == the same annealOneStep calls (bit-exact)."""
    rng = np.random.default_rng(8)
    W = rand_sym(rng, 96)
    G = [5.0 * 0.9 ** k for k in range(20)]
    res = []
    for batched in (False, True):
        a = sq.cuda.dense_graph_annealer(W, n_trotters=12)
        a.seed(5)
        a.prepare()
        a.randomize_spin()
        if batched:
            a.anneal(np.array(G, np.float32), 20.0)
        else:
            for g in G:
                a.anneal_one_step(g, 20.0)
        res.append((np.array(a.get_q()), a.get_E64()))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


# ------------------------------------------------------ known-answer anneals
def _anneal(a, sq):
    a.prepare()
    a.randomize_spin()
    algo = a.get_preferences()["algorithm"]
    if algo in ("sa_naive", "sa_coloring"):
        Ginit, Gfin, beta = 10., 0.02, 1.
    else:
        Ginit, Gfin, beta = 5., 0.02, 1. / 0.03
    nSteps = 100
    tau = math.exp(math.log(Gfin / Ginit) / nSteps)
    G = Ginit
    for _ in range(nSteps):
        a.anneal_one_step(G, beta)
        G *= tau


@pytest.mark.parametrize("algo,m", [("naive", 4), ("coloring", 4), ("default", 4), ("sa_naive", 1),
                                    ("default", 1)])
def test_dense_anneal_known_answers(sq, algo, m):
    N = 10
    a = sq.cuda.dense_graph_annealer(np.ones((N, N), np.float32), sq.minimize, n_trotters=m, algorithm=algo)
    a.seed(42)
    _anneal(a, sq)
    assert a.get_E().min() == 0
    a = sq.cuda.dense_graph_annealer(-np.ones((N, N), np.float32), sq.maximize, n_trotters=m, algorithm=algo)
    a.seed(43)
    _anneal(a, sq)
    assert a.get_E().max() == 0
    h, J, c = (v.astype(np.float32) if hasattr(v, "astype") else v for v in
               _py_hamiltonian(np.ones((N, N))))
    a = sq.cuda.dense_graph_annealer(n_trotters=m)
    a.set_hamiltonian(h, J, c)
    a.set_preferences(n_trotters=m, algorithm=algo)
    a.seed(44)
    _anneal(a, sq)
    assert a.get_E().max() == 0


def _py_hamiltonian(W):
    from oracle import oracle_ctypes
    return oracle_ctypes.dg_hamiltonian(W)


@pytest.mark.parametrize("algo", ["naive", "coloring", "default", "sa_coloring", "sa_naive"])
def test_bipartite_anneal_known_answers(sq, algo):
    N0, N1, m = 10, 8, 6
    ones = lambda *s: np.ones(s, np.float32)
    a = sq.cuda.bipartite_graph_annealer(ones(N0), ones(N1), ones(N1, N0), sq.minimize, n_trotters=m,
                                         algorithm=algo)
    a.seed(7)
    _anneal(a, sq)
    assert a.get_E().min() == 0
    a = sq.cuda.bipartite_graph_annealer(-ones(N0), -ones(N1), -ones(N1, N0), sq.maximize, n_trotters=m,
                                         algorithm=algo)
    a.seed(8)
    _anneal(a, sq)
    assert a.get_E().max() == 0


# ----------------------------------------------------------- solver API
def test_calling_sequence_and_state(sq):
    rng = np.random.default_rng(1)
    N, m = 200, 100
    a = sq.cuda.dense_graph_annealer(rand_sym(rng, N), n_trotters=m, algorithm=sq.algorithm.default)
    a.seed(0)
    a.prepare()
    a.randomize_spin()
    a.anneal_one_step(1, 1)
    a.calculate_E()
    a.get_system_E(1, 1)
    a.make_solution()
    assert len(a.get_E()) == m and len(a.get_x()) == m and len(a.get_q()) == m
    assert a.get_problem_size() == N
    h, J, c = a.get_hamiltonian()
    assert h.shape == (N,) and J.shape == (N, N)
    b = sq.cuda.dense_graph_annealer(rand_sym(rng, 10), n_trotters=10)
    with pytest.raises(RuntimeError):
        b.anneal_one_step(0., 0.)


def test_set_q_roundtrip(sq):
    rng = np.random.default_rng(2)
    N, m = 100, 100
    a = sq.cuda.dense_graph_annealer(rand_sym(rng, N), n_trotters=m)
    a.prepare()
    qin = (2 * rng.integers(0, 2, N) - 1).astype(np.int8)
    a.set_q(qin)
    assert all(np.array_equal(qin, q) for q in a.get_q())
    qs = [(2 * rng.integers(0, 2, 5) - 1).astype(np.int8) for _ in range(2)]
    b = sq.cuda.dense_graph_annealer(rand_sym(rng, 5), n_trotters=2)
    b.set_qset(qs)
    assert all(np.array_equal(x, y) for x, y in zip(qs, b.get_q()))


def _spin_energy_ref(qset, G, beta):
    m = len(qset)
    E = 0.
    for im in range(m):
        E += np.sum(qset[im].astype(np.float64) * qset[(im + 1) % m])
    return E * 1. / (2 * beta) * np.log(1 / np.tanh(G * beta / m))


def test_get_system_E(sq):
    G, beta = 0.01, 1. / 0.05
    N, m = 10, 5
    rng = np.random.default_rng(4)
    a = sq.cuda.dense_graph_annealer(rand_sym(rng, N), n_trotters=m, algorithm=sq.algorithm.sa_default)
    a.prepare()
    qset = (2 * rng.integers(0, 2, (m, N)) - 1).astype(np.int8)
    a.set_qset(qset)
    assert np.allclose(a.get_system_E(G, beta), np.mean(a.get_E()), atol=1e-5)
    a = sq.cuda.dense_graph_annealer(np.ones((N, N), np.float32), n_trotters=m)
    a.prepare()
    for sign in (1, -1):
        a.set_q(sign * np.ones(N, np.int8))
        ref = np.mean(a.get_E()) + _spin_energy_ref(a.get_q(), G, beta)
        assert np.allclose(a.get_system_E(G, beta), ref, rtol=1e-5, atol=1e-4)


# -------------------------------------------------------- brute force
@pytest.mark.parametrize("name", ["int12", "int16", "int16max", "ex8", "pos8min", "neg8min", "pos8max", "r10"])
def test_dense_bf_golden(sq, golden, name):
    W = golden["bf_%s_W" % name].astype(np.float32)
    om = sq.maximize if int(golden["bf_%s_om" % name]) else sq.minimize
    s = sq.cuda.dense_graph_bf_searcher(W, om)
    s.search()
    E, x = s.get_E(), np.array(s.get_x())
    assert np.allclose(E, golden["bf_%s_E" % name][0], atol=1e-6)
    assert np.array_equal(x, golden["bf_%s_x" % name])


def test_dense_bf_minimum_run_vs_cpu_reference(sq, orc, golden):
    """sqaodc/tests/CUDADenseGraphBFSolverTest.cpp:218-247 at N = 16, and integer
    W uniform in [-8, 8] at N = 20: Emin and argmin set bit-exact."""
    W16 = golden["bf_int16_W"].astype(np.float32)
    rng = np.random.default_rng(0)
    U = rng.integers(-8, 9, (20, 20))
    W20 = (np.triu(U) + np.triu(U, 1).T).astype(np.float32)
    for W in (W16, W20):
        E_ref, xs_ref = orc.dg_bf_search_ref(W, n_workers=0)
        s = sq.cuda.dense_graph_bf_searcher(W)
        s.search()
        assert s.get_E()[0] == E_ref
        assert np.array_equal(np.array(s.get_x()), orc.unpack_bits(xs_ref, W.shape[0]))


def test_dense_bf_search_range_tiles(sq, orc):
    """search_range over small tiles == search(), including ties and the tile cap."""
    rng = np.random.default_rng(9)
    U = rng.integers(-1, 2, (14, 14))
    W = (np.triu(U) + np.triu(U, 1).T).astype(np.float32)
    s1 = sq.cuda.dense_graph_bf_searcher(W, tile_size=256)
    s1.search()
    s2 = sq.cuda.dense_graph_bf_searcher(W, tile_size=256)
    s2.prepare()
    n = 0
    while not s2.search_range():
        n += 1
    s2.make_solution()
    assert n == (1 << 14) // 256 - 1
    assert np.array_equal(np.array(s1.get_x()), np.array(s2.get_x()))
    E_ref, xs_ref = orc.dg_bf_search_range(W, 0, 0, 1 << 14, 256)
    assert s1.get_E()[0] == E_ref
    assert np.array_equal(np.array(s1.get_x()), orc.unpack_bits(xs_ref, 14))
    # all-zero W: every state ties; the first tile_size states are returned
    z = sq.cuda.dense_graph_bf_searcher(np.zeros((12, 12), np.float32), tile_size=512)
    z.search()
    assert len(z.get_x()) == 512
    assert np.array_equal(np.array(z.get_x()), orc.unpack_bits(np.arange(512), 12))


def test_bipartite_bf_golden(sq, orc, golden):
    g = golden
    s = sq.cuda.bipartite_graph_bf_searcher(g["bbf_b0"], g["bbf_b1"], g["bbf_W"])
    s.search()
    assert np.allclose(s.get_E()[0], g["bbf_E"][0], atol=1e-6)
    xs = s.get_x()
    assert np.array_equal(np.array([p[0] for p in xs]), g["bbf_x0"])
    assert np.array_equal(np.array([p[1] for p in xs]), g["bbf_x1"])
    # integer problem with ties, against the reference CPU searcher
    rng = np.random.default_rng(6)
    b0 = rng.integers(-2, 3, 9).astype(np.float32)
    b1 = rng.integers(-2, 3, 7).astype(np.float32)
    W = rng.integers(-2, 3, (7, 9)).astype(np.float32)
    E_ref, pairs = orc.bg_bf_search_sorted(b0, b1, W)
    s = sq.cuda.bipartite_graph_bf_searcher(b0, b1, W, tile_size_0=256, tile_size_1=256)
    s.search()
    got = sorted((bits_to_int(p[0]), bits_to_int(p[1])) for p in s.get_x())
    assert s.get_E()[0] == E_ref
    assert got == sorted((int(a), int(b)) for a, b in pairs)
    s2 = sq.cuda.bipartite_graph_bf_searcher(b0, b1, W, tile_size_0=256, tile_size_1=256)
    s2.prepare()
    while not s2.search_range():
        pass
    s2.make_solution()
    assert [(tuple(a), tuple(b)) for a, b in s2.get_x()] == [(tuple(a), tuple(b)) for a, b in s.get_x()]


def test_dense_bf_shards_merge_to_whole_search(sq):
    """Sub-range searches (the shards of a multi-GPU search) merged on the host
    equal one search of the whole range: FP64 minimum and minimiser list."""
    from sqaod_gb300 import shard
    rng = np.random.default_rng(3)
    U = np.triu(rng.integers(-8, 9, (20, 20)))
    W = (U + np.triu(U, 1).T).astype(np.float32)
    for optimize in (sq.minimize, sq.maximize):
        parts = [shard.gpu_shard_search(W, optimize, *shard.shard_range(1 << 20, r, 3), 1024) for r in range(3)]
        E, xs = shard.merge_shards(parts, 1024)
        s = sq.cuda.dense_graph_bf_searcher(W, optimize, tile_size=1024)
        s.search()
        E_all = s.get_E64()
        assert (-E if optimize is sq.maximize else E) == E_all
        assert xs.tolist() == [shard.pack_bits(x) for x in s.get_x()]
    s = sq.cuda.dense_graph_bf_searcher(W)
    s.prepare()
    s.search_subrange(16, 64)
    with pytest.raises(RuntimeError):  # ranges must ascend
        s.search_subrange(0, 8)


def test_bf_known_answers(sq):
    N = 8
    for W, om, E, x in ((np.ones((N, N)), sq.minimize, 0., 0), (-np.ones((N, N)), sq.minimize, -64., 1),
                        (np.ones((N, N)), sq.maximize, 64., 1), (-np.ones((N, N)), sq.maximize, 0., 0)):
        s = sq.cuda.dense_graph_bf_searcher(W.astype(np.float32), om)
        s.search()
        assert s.get_E()[0] == E and np.all(np.array(s.get_x()) == x)
    s = sq.cuda.dense_graph_bf_searcher(np.ones((4, 4), np.float32), sq.maximize)
    s.prepare()
    s.search()
    assert len(s.get_E()) == 1 and s.get_E()[0] == 16
