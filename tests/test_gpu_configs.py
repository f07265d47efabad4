"""Parity at the benchmarked configurations themselves, through the C ABI.

- dense N = 4096, m = 256 (the headline instance, the bench's own W): two
  8-step sweep launches with the field refresh between them, early (G = 5) and
  late (G ~ 0.05) in the 619-step schedule, replayed against FP64 over the
  same Philox stream (resident FP64 fields, oracle orc_dg_replay_steps);
- dense N = 128, m = 16: the whole 619-step anneal replayed, and the final
  FP64 energies;
- bipartite N0 = N1 = 1024, m = 64: 8 steps early and late, replayed;
- brute-force N = 32 (2^32 states, integer W in [-8, 8], the bench's W): Emin
  and the minimiser list against the exact integer enumeration, and N = 28
  against the restated reference CPU searcher itself;
- ground-state success probability at N = 24 against the reference CPU
  coloring annealer, on a schedule short enough that neither arm saturates.

Replay rule (the same as tests/test_gpu_parity.py): a device decision may
differ from the FP64 decision only where the FP64 acceptance margin
|min(1, exp(-rate dE)) - u| is below 1e-6; those trials are counted and
printed.
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402  (the benchmark's own instance generators)

MARGIN_TOL = 1e-6
BETA = 50.0


@pytest.fixture(scope="module")
def sq():
    import sqaod_gb300
    return sqaod_gb300


def schedule():
    """G = 5 * 0.99^k while G > 0.01: the 619 steps of the plain-solver configs."""
    out, G = [], 5.0
    while G > 0.01:
        out.append(G)
        G *= 0.99
    return np.array(out, np.float32)


def _replay_dense(sq, orc, N, m, algo, start, n_steps, seed=0):
    W = bench.problem(N)
    a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm=algo)
    a.seed(seed)
    a.prepare()
    a.randomize_spin()
    G = schedule()
    if start:
        a.anneal(G[:start], BETA)
    q = np.array(a.get_q())
    h, J, c = a.get_hamiltonian()
    assert np.array_equal(J, J.T) and not np.diag(J).any()
    a.set_trace(True)
    _, step0 = a.get_rng_state()
    Gs = G[start:start + n_steps]
    a.anneal(Gs, BETA)
    words = (N * m + 31) // 32
    trace = a.get_trace(words * len(Gs))
    code = {"coloring": orc.ALGO_COLORING, "sa_naive": orc.ALGO_SA_NAIVE, "naive": orc.ALGO_NAIVE}[algo]
    q_host, st = orc.dg_replay_steps(h, J, m, code, seed, step0, Gs, BETA, q, trace, MARGIN_TOL)
    print("N=%d m=%d %s steps %d..%d (G %.3g..%.3g): %s" % (N, m, algo, start, start + len(Gs) - 1,
                                                          Gs[0], Gs[-1], st))
    return a, q_host, st, (h, J, c)


@pytest.mark.parametrize("algo,start", [("coloring", 0), ("coloring", 456), ("sa_naive", 0)])
def test_headline_dense_replays_fp64(sq, orc, algo, start):
    """N = 4096, m = 256: 16 steps = two 8-step sweep launches with the field
    refresh between them (the anneal starts right after a refresh and 456 is a
    multiple of 8), at the start of the schedule (G = 5) and near its end
    (G = 0.051)."""
    a, q_host, st, _ = _replay_dense(sq, orc, 4096, 256, algo, start, 16)
    assert st["n_trials"] == 16 * 4096 * 256
    assert st["n_accept"] > 0
    assert np.array_equal(np.array(a.get_q()), q_host), "device spins differ from the replayed trace"
    assert st["n_mismatch"] == st["n_mismatch_small"], st


def test_c1_dense_whole_anneal_replays_fp64(sq, orc):
    """N = 128, m = 16: every one of the 619 steps of the anneal replays, and
    the returned FP64 energies are those of the final spins."""
    G = schedule()
    a, q_host, st, (h, J, c) = _replay_dense(sq, orc, 128, 16, "coloring", 0, len(G))
    assert st["n_trials"] == len(G) * 128 * 16
    q = np.array(a.get_q())
    assert np.array_equal(q, q_host)
    assert st["n_mismatch"] == st["n_mismatch_small"], st
    a.make_solution()
    E = a.get_E64()
    # the device keeps h, J in fp32 (get_hamiltonian) and the constant c in FP64
    h64, J64, c64 = orc.dg_hamiltonian(bench.problem(128))
    E_ref = orc.dg_energy_ising(h, J, c64, q)
    assert np.max(np.abs(E - E_ref)) <= 1e-11 * max(1.0, np.max(np.abs(E_ref)))
    # within 1e-5 of the all-FP64 Hamiltonian of the fp32 W as well
    E_ref64 = orc.dg_energy_ising(h64, J64, c64, q)
    assert np.max(np.abs(E - E_ref64)) <= 1e-5 * max(1.0, np.max(np.abs(E_ref64)))
    print("C1 min E %.6f" % E.min())


@pytest.mark.parametrize("algo,start", [("coloring", 0), ("coloring", 456), ("sa_coloring", 0)])
def test_c2_bipartite_replays_fp64(sq, orc, algo, start):
    """N0 = N1 = 1024, m = 64, the bench's instance: 8 steps early and late."""
    N0 = N1 = 1024
    m = 64
    rs = np.random.RandomState(0)
    b0 = rs.uniform(-1, 1, N0).astype(np.float32)
    b1 = rs.uniform(-1, 1, N1).astype(np.float32)
    W = rs.uniform(-1, 1, (N1, N0)).astype(np.float32)
    a = sq.cuda.bipartite_graph_annealer(b0, b1, W, n_trotters=m, algorithm=algo)
    seed = 7
    a.seed(seed)
    a.prepare()
    a.randomize_spin()
    G = schedule()
    if start:
        a.anneal(G[:start], BETA)
    pairs = a.get_q()
    q0 = np.array([p[0] for p in pairs])
    q1 = np.array([p[1] for p in pairs])
    h0, h1, J, c = a.get_hamiltonian()
    a.set_trace(True)
    code = {"coloring": orc.ALGO_COLORING, "sa_coloring": orc.ALGO_SA_COLORING}[algo]
    tot = {}
    for s in range(8):
        _, step = a.get_rng_state()
        a.anneal_one_step(float(G[start + s]), BETA)
        trace = a.get_trace((m * (N0 + N1) + 31) // 32)
        q0, q1, st = orc.bg_replay(h0, h1, J, m, code, seed, step, float(G[start + s]), BETA, q0, q1, trace,
                                   MARGIN_TOL)
        pairs = a.get_q()
        assert np.array_equal(np.array([p[0] for p in pairs]), q0)
        assert np.array_equal(np.array([p[1] for p in pairs]), q1)
        for k, v in st.items():
            tot[k] = max(tot.get(k, 0), v) if k == "max_mismatch_margin" else tot.get(k, 0) + v
    print("bipartite %s from step %d: %s" % (algo, start, tot))
    assert tot["n_trials"] == 8 * m * (N0 + N1)
    assert tot["n_mismatch"] == tot["n_mismatch_small"], tot


def test_bipartite_tensor_core_fields_replay_fp64(sq, orc):
    """A bipartite annealer whose half-step fields come from the tensor cores
    (N0 = N1 = 2048, m = 256: 64 output tiles per half step), replayed against
    FP64 over two steps."""
    from sqaod_gb300 import _lib
    N0 = N1 = 2048
    m = 256
    assert _lib.lib().sq103_bipartite_refresh_uses_tc(N0, N1, m) == 1
    rs = np.random.RandomState(5)
    b0 = rs.uniform(-1, 1, N0).astype(np.float32)
    b1 = rs.uniform(-1, 1, N1).astype(np.float32)
    W = rs.uniform(-1, 1, (N1, N0)).astype(np.float32)
    a = sq.cuda.bipartite_graph_annealer(b0, b1, W, n_trotters=m, algorithm="coloring")
    seed = 11
    a.seed(seed)
    a.prepare()
    a.randomize_spin()
    pairs = a.get_q()
    q0 = np.array([p[0] for p in pairs])
    q1 = np.array([p[1] for p in pairs])
    h0, h1, J, c = a.get_hamiltonian()
    a.set_trace(True)
    tot = {}
    for G in (2.0, 0.05):
        _, step = a.get_rng_state()
        a.anneal_one_step(G, BETA)
        trace = a.get_trace((m * (N0 + N1) + 31) // 32)
        q0, q1, st = orc.bg_replay(h0, h1, J, m, orc.ALGO_COLORING, seed, step, G, BETA, q0, q1, trace, MARGIN_TOL)
        pairs = a.get_q()
        assert np.array_equal(np.array([p[0] for p in pairs]), q0)
        assert np.array_equal(np.array([p[1] for p in pairs]), q1)
        for k, v in st.items():
            tot[k] = max(tot.get(k, 0), v) if k == "max_mismatch_margin" else tot.get(k, 0) + v
    print("bipartite on tensor-core fields: %s" % tot)
    assert tot["n_mismatch"] == tot["n_mismatch_small"], tot


@pytest.mark.parametrize("optimize", ["minimize", "maximize"])
def test_c3_bf_n32_exact(sq, orc, optimize):
    """All 2^32 states of the bench's N = 32 integer QUBO: Emin and every
    minimiser (ascending, first tile_size) identical to the exact integer
    enumeration, which equals the reference CPU searcher on integer W."""
    W = bench.bf_problem(32)
    om = getattr(sq, optimize)
    s = sq.cuda.dense_graph_bf_searcher(W, om)
    s.search()
    tile = s.get_preferences()["tile_size"]
    E_ref, xs_ref, count = orc.dg_bf_search_exact_int(W, 1 if optimize == "maximize" else 0, cap=tile)
    xs = [int("".join(str(int(b)) for b in x), 2) for x in s.get_x()]
    print("N=32 %s: Emin %g, %d minimiser(s) %s" % (optimize, E_ref, count, xs_ref[:4]))
    assert float(s.get_E()[0]) == E_ref
    assert xs == xs_ref.tolist()


def test_c3_bf_n28_reference_searcher(sq, orc):
    """N = 28 (where the CPU baseline is timed), against the restated reference
    CPU searcher itself (tile sweep, tie / cap / merge rules)."""
    W = bench.bf_problem(28)
    s = sq.cuda.dense_graph_bf_searcher(W, tile_size=1024)
    s.search()
    E_ref, xs_ref = orc.dg_bf_search_ref(W, 0, tile_size=1024)
    xs = [int("".join(str(int(b)) for b in x), 2) for x in s.get_x()]
    assert float(s.get_E()[0]) == E_ref
    assert xs == xs_ref.tolist()


def test_success_probability_matches_reference_cpu(sq, orc):
    """Ground-state success probability of the GPU coloring annealer against the
    reference CPU coloring annealer at N = 24, m = 8, beta = 50, on the 3-step
    geometric schedule G = 5 -> 0.22 -> 0.01, where both arms land near 0.57
    (the full 619-step schedule solves every seed on both arms).  64 seeds give
    a standard error of about 9 points on the difference at p ~ 0.5, so the
    +-5-point criterion is asserted over 2048 seeds per arm (standard error
    1.6 points); the first 64 seeds are printed too.  A CPU arm with m = 4 in
    place of 8 lands 20 points lower, so the check separates a wrong
    annealer."""
    N, m, seeds = 24, 8, 2048
    np.random.seed(0)
    W = sq.generate_random_symmetric_W(N, -1., 1., np.float64).astype(np.float32)
    s = sq.cuda.dense_graph_bf_searcher(W)
    s.search()
    E0 = float(s.get_E()[0])
    G = np.array([5.0 * (0.01 / 5.0) ** (k / 2.0) for k in range(3)], np.float32)
    a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm="coloring")
    gpu = np.zeros(seeds, bool)
    for seed in range(seeds):
        a.seed(seed)
        a.prepare()
        a.randomize_spin()
        a.anneal(G, BETA)
        gpu[seed] = a.get_E().min() <= E0 + 1e-4
    h, J, c = orc.dg_hamiltonian(W)

    def cpu_arm(mm, n):
        hits = np.zeros(n, bool)
        for seed in range(n):
            r = orc.DenseAnnealerRef(h, J, c, mm, n_workers=1)
            r.seed(seed)
            r.randomize_spin()
            for g in G:
                r.anneal_one_step(orc.ALGO_COLORING, float(g), BETA)
            hits[seed] = r.get_E().min() <= E0 + 1e-4
        return hits

    cpu = cpu_arm(m, seeds)
    wrong = cpu_arm(4, 512).mean()
    p_gpu, p_cpu = gpu.mean(), cpu.mean()
    print("success probability over %d seeds: gpu %.3f cpu %.3f (first 64 seeds: gpu %.3f cpu %.3f); "
          "CPU with m = 4: %.3f" % (seeds, p_gpu, p_cpu, gpu[:64].mean(), cpu[:64].mean(), wrong))
    assert 0.2 <= p_cpu <= 0.8 and 0.2 <= p_gpu <= 0.8, (p_gpu, p_cpu)
    assert abs(p_gpu - p_cpu) <= 0.05, (p_gpu, p_cpu)
    assert abs(wrong - p_cpu) > 0.05, (wrong, p_cpu)
