"""Pins the CPU oracle before it is trusted (CPU only).

- MT19937 and the AVX2-order dot against the reference's own Random.cpp /
  Dot_SIMD.cpp compiled from source (oracle/_ref; skipped where it cannot be
  built) and against published known answers;
- Philox4x32-10 against the Random123 known-answer vectors;
- formulas and brute-force results against golden vectors generated from the
  reference's numpy backend (tests/golden/make_golden.py) and the reference
  tests' known answers.
"""
import ctypes
import os

import numpy as np
import pytest


def test_philox_known_answers(orc):
    # Random123 kat_vectors, philox4x32_10
    assert list(orc.philox([0, 0, 0, 0], [0, 0])) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert list(orc.philox([0xffffffff] * 4, [0xffffffff] * 2)) == [
        0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert list(orc.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                           [0xa4093822, 0x299f31d0])) == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_mt19937_known_answer(orc):
    # MT19937 reference output for init_genrand(5489)
    assert orc.mt_stream(5489, 1)[0] == 3499211612


def _ref_lib():
    from oracle import build
    path = build.build_ref()
    if path is None:
        pytest.skip("reference sources not present or host is not x86_64")
    return ctypes.CDLL(path)


def test_mt19937_matches_reference_source(orc):
    ref = _ref_lib()
    for seed in (0, 1, 17, 5489, 2 ** 40 + 3):
        a = np.zeros(5000, np.uint32)
        ref.ref_mt_stream(ctypes.c_ulonglong(seed), 5000, a.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(a, orc.mt_stream(seed, 5000))


def test_dot_matches_reference_source(orc):
    ref = _ref_lib()
    ref.ref_dot_avx2.restype = ctypes.c_float
    rng = np.random.default_rng(1)
    for N in (1, 7, 16, 31, 128, 1000, 4096):
        a = rng.standard_normal(N).astype(np.float32)
        b = rng.choice([-1.0, 1.0], N).astype(np.float32)
        r = ref.ref_dot_avx2(a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p), N)
        assert np.float32(r).tobytes() == np.float32(orc.dot_ref(a, b)).tobytes()


@pytest.mark.parametrize("name", ["ex8", "r16", "r100"])
def test_dense_hamiltonian_golden(orc, golden, name):
    W = golden["dg_%s_W" % name]
    h, J, c = orc.dg_hamiltonian(W)
    assert np.allclose(h, golden["dg_%s_h" % name], rtol=0, atol=1e-12)
    assert np.allclose(J, golden["dg_%s_J" % name], rtol=0, atol=1e-12)
    assert abs(c - golden["dg_%s_c" % name]) < 1e-10


def test_dense_energies_golden(orc, golden):
    W, X = golden["dg_r8_W"], golden["dg_r8_X"]
    assert np.allclose(orc.dg_energy_qubo(W, X), golden["dg_r8_E"], atol=1e-12)
    h, J, c = orc.dg_hamiltonian(W)
    Q = (2 * X - 1).astype(np.int8)
    Ei = orc.dg_energy_ising(h, J, c, Q)
    assert np.allclose(Ei, golden["dg_r8_Eising"], atol=1e-12)
    # QUBO <-> Ising identity: E_qubo(x) == E_ising(2x - 1)
    assert np.allclose(Ei, golden["dg_r8_E"], atol=1e-12)


def test_ising_identity_and_known_answers(orc):
    # -sum(h) + sum(J) + c == 0 (sqaodpy/tests/test_dense_graph_formulas.py:56-80)
    rng = np.random.default_rng(2)
    W = rng.uniform(-1, 1, (20, 20))
    W = np.triu(W) + np.triu(W, 1).T
    h, J, c = orc.dg_hamiltonian(W)
    assert abs(-h.sum() + J.sum() + c) < 1e-10
    # W = ones, q = +1 -> E = N^2 (sqaodpy/tests/test_dense_graph_annealer.py:154-165)
    N = 8
    h, J, c = orc.dg_hamiltonian(np.ones((N, N)))
    assert orc.dg_energy_ising(h, J, c, np.ones((1, N), np.int8))[0] == N * N
    # all -1 spins -> E = 0 (test_min_energy)
    assert abs(orc.dg_energy_ising(h, J, c, -np.ones((1, N), np.int8))[0]) < 1e-12


def test_bipartite_formulas_golden(orc, golden):
    g = golden
    h0, h1, J, c = orc.bg_hamiltonian(g["bg_b0"], g["bg_b1"], g["bg_W"])
    assert np.allclose(h0, g["bg_h0"], atol=1e-12) and np.allclose(h1, g["bg_h1"], atol=1e-12)
    assert np.allclose(J, g["bg_J"], atol=1e-12) and abs(c - g["bg_c"]) < 1e-10
    E = orc.bg_energy_qubo(g["bg_b0"], g["bg_b1"], g["bg_W"], g["bg_x0"], g["bg_x1"])
    assert np.allclose(E, g["bg_E"], atol=1e-12)
    E2 = orc.bg_energy_qubo_2d(g["bg_b0"], g["bg_b1"], g["bg_W"], g["bg_x0"][:7], g["bg_x1"][:7])
    assert np.allclose(E2, g["bg_E2d"], atol=1e-12)
    q0 = (2 * g["bg_x0"] - 1).astype(np.int8)
    q1 = (2 * g["bg_x1"] - 1).astype(np.int8)
    assert np.allclose(orc.bg_energy_ising(h0, h1, J, c, q0, q1), g["bg_Eising"], atol=1e-12)
    # W = ones, b = ones, q = +1 -> N0*N1 + N0 + N1 (test_bipartite_graph_annealer.py:170-182)
    N0, N1 = 4, 4
    h0, h1, J, c = orc.bg_hamiltonian(np.ones(N0), np.ones(N1), np.ones((N1, N0)))
    e = orc.bg_energy_ising(h0, h1, J, c, np.ones((1, N0), np.int8), np.ones((1, N1), np.int8))[0]
    assert e == N0 * N1 + N0 + N1


@pytest.mark.parametrize("name", ["int12", "int16", "int16max", "ex8", "pos8min", "neg8min",
                                  "pos8max", "r10"])
def test_dense_bf_golden(orc, golden, name):
    W = golden["bf_%s_W" % name]
    om = int(golden["bf_%s_om" % name])
    for workers in (1, 3):
        E, xs = orc.dg_bf_search_ref(W, om=om, n_workers=workers)
        assert np.allclose(E, golden["bf_%s_E" % name][0], atol=1e-6)
        X = orc.unpack_bits(xs, W.shape[0])
        assert np.array_equal(X, golden["bf_%s_x" % name])


def test_dense_bf_tie_cap_semantics(orc):
    # W = 0: every state ties; the reference keeps tileSize solutions, sorted
    W = np.zeros((12, 12), np.float32)
    E, xs = orc.dg_bf_search_ref(W, tile_size=256, n_workers=1)
    assert E == 0 and len(xs) == 256 and np.array_equal(xs, np.arange(256))
    E2, xs2 = orc.dg_bf_search_range(W, 0, 0, 4096, 100)
    assert len(xs2) == 100 and np.array_equal(xs2, np.arange(100))


def test_bipartite_bf_golden(orc, golden):
    g = golden
    E, pairs = orc.bg_bf_search_ref(g["bbf_b0"], g["bbf_b1"], g["bbf_W"], n_workers=2)
    assert np.allclose(E, g["bbf_E"][0], atol=1e-6)
    x0 = orc.unpack_bits(pairs[:, 0], len(g["bbf_b0"]))
    x1 = orc.unpack_bits(pairs[:, 1], len(g["bbf_b1"]))
    assert np.array_equal(x0, g["bbf_x0"]) and np.array_equal(x1, g["bbf_x1"])
    E2, pairs2 = orc.bg_bf_search_sorted(g["bbf_b0"], g["bbf_b1"], g["bbf_W"])
    assert E2 == E and np.array_equal(pairs2, pairs)


def test_reference_annealers_reach_known_answers(orc):
    # W = ones, N = 10, m = 4 anneals must reach E == 0
    # (sqaodpy/tests/test_dense_graph_annealer.py:180-262)
    N, m = 10, 4
    h, J, c = orc.dg_hamiltonian(np.ones((N, N)))
    for algo in (orc.ALGO_NAIVE, orc.ALGO_COLORING):
        a = orc.DenseAnnealerRef(h, J, c, m, n_workers=2)
        a.seed(0)
        a.randomize_spin()
        G, beta = 5.0, 1.0 / 0.03
        tau = np.exp(np.log(0.02 / 5.0) / 100)
        for _ in range(100):
            a.anneal_one_step(algo, G, beta)
            G *= tau
        assert a.get_E().min() == 0
    h0, h1, Jb, cb = orc.bg_hamiltonian(np.ones(10), np.ones(8), np.ones((8, 10)))
    for algo in (orc.ALGO_NAIVE, orc.ALGO_COLORING, orc.ALGO_SA_COLORING):
        a = orc.BipartiteAnnealerRef(h0, h1, Jb, cb, 6, n_workers=2)
        a.seed(1)
        a.randomize_spin()
        G, beta = (10.0, 1.0) if algo == orc.ALGO_SA_COLORING else (5.0, 1.0 / 0.03)
        Gfin = 0.02
        tau = np.exp(np.log(Gfin / G) / 100)
        for _ in range(100):
            a.anneal_one_step(algo, G, beta)
            G *= tau
        assert abs(a.get_E().min()) < 1e-9


def test_replay_self_consistency(orc):
    """A replay fed its own decisions reports no mismatch."""
    rng = np.random.default_rng(3)
    N, m = 24, 6
    W = rng.uniform(-1, 1, (N, N))
    W = np.triu(W) + np.triu(W, 1).T
    h, J, c = orc.dg_hamiltonian(W)
    q = orc.gpu_randomize(7, 0, 0, m, N)
    assert set(np.unique(q)) <= {-1, 1}
    # an all-accept trace makes every decision follow the device; mismatches
    # are then exactly the FP64 rejections, so n_mismatch == n_trials - host accepts
    trace = np.full((N * m + 31) // 32, 0xffffffff, np.uint32)
    q2, st = orc.dg_replay(h, J, m, orc.ALGO_COLORING, 7, 1, 1.0, 10.0, q, trace)
    assert st["n_trials"] == N * m and st["n_accept"] == N * m


@pytest.mark.parametrize("algo", ["ALGO_COLORING", "ALGO_NAIVE", "ALGO_SA_NAIVE"])
@pytest.mark.parametrize("N,m", [(40, 6), (33, 7)])
def test_replay_steps_equals_per_step_replay(orc, algo, N, m):
    """The resident-FP64-field replay (used at the benchmark size) takes the same
    decisions and reports the same statistics as the direct-dot replay, over
    several steps of a random device trace (about 6 % accepts)."""
    rng = np.random.default_rng(N * m)
    W = rng.uniform(-1, 1, (N, N))
    W = np.triu(W) + np.triu(W, 1).T
    h, J, c = orc.dg_hamiltonian(W)
    h, J = h.astype(np.float32), J.astype(np.float32)
    assert np.array_equal(J, J.T) and not np.diag(J).any()
    q0 = orc.gpu_randomize(11, 0, 0, m, N)
    G = np.array([3.0, 1.0, 0.3, 0.05], np.float32)
    beta = np.array([10.0, 20.0, 30.0, 50.0], np.float32)
    words = (N * m + 31) // 32
    bits = rng.random((len(G), words * 32)) < 0.06
    trace = np.packbits(bits, axis=1, bitorder="little").view(np.uint32)
    a = getattr(orc, algo)
    q, tot = q0.copy(), {}
    for s in range(len(G)):
        q, st = orc.dg_replay(h, J, m, a, 11, 5 + s, float(G[s]), float(beta[s]), q, trace[s])
        for k, v in st.items():
            tot[k] = max(tot.get(k, 0), v) if k == "max_mismatch_margin" else tot.get(k, 0) + v
    q2, st2 = orc.dg_replay_steps(h, J, m, a, 11, 5, G, beta, q0, trace)
    assert np.array_equal(q, q2)
    assert tot["n_trials"] == st2["n_trials"] == len(G) * N * m
    for k in ("n_accept", "n_mismatch", "n_mismatch_small", "n_small_margin"):
        assert tot[k] == st2[k], (k, tot, st2)
    assert tot["n_mismatch"] > 0  # a random trace disagrees with FP64 somewhere


@pytest.mark.parametrize("N,om,lo,hi", [(16, 0, -8, 9), (20, 1, -8, 9), (18, 0, -1, 2), (13, 1, 0, 2)])
def test_exact_int_search_equals_reference_searcher(orc, N, om, lo, hi):
    """The Gray-code integer search (the checker at N = 32) gives the restated
    reference CPU searcher's minimum and minimiser list, ties and the
    tileSize cap included (the narrow ranges make many minimisers)."""
    rng = np.random.default_rng(N + om)
    U = np.triu(rng.integers(lo, hi, (N, N)))
    W = (U + np.triu(U, 1).T).astype(np.float32)
    for tile in (1024, 16):
        E_ref, xs_ref = orc.dg_bf_search_ref(W, om, tile_size=tile)
        E, xs, count = orc.dg_bf_search_exact_int(W, om, cap=tile)
        assert E == E_ref and xs.tolist() == xs_ref.tolist(), (E, E_ref, count)
        assert count >= len(xs)
    assert orc.dg_bf_search_exact_int(W, om, cap=1 << 16)[2] == count


def test_exact_int_search_rejects_non_integer(orc):
    W = np.full((8, 8), 0.5, np.float32)
    with pytest.raises(ValueError):
        orc.dg_bf_search_exact_int(W)
