"""Checkpoint / resume of the annealers: an anneal interrupted after any step,
saved with numpy.savez, and restored into a fresh annealer ends with exactly
the spins and FP64 energies of the uninterrupted anneal."""
import io

import numpy as np
import pytest

import sqaod_gb300 as sq

pytestmark = pytest.mark.gpu
BETA = 50.


def schedule(n):
    return [5. * 0.9 ** i for i in range(n)]


def sym_W(N, seed):
    rng = np.random.default_rng(seed)
    W = rng.uniform(-1, 1, (N, N))
    return (np.triu(W) + np.triu(W, 1).T).astype(np.float32)


def through_file(state):
    buf = io.BytesIO()
    np.savez(buf, **state)
    buf.seek(0)
    with np.load(buf) as z:
        return {k: z[k] for k in z.files}


def dense(W, m, algo, seed=7):
    a = sq.cuda.dense_graph_annealer(W, sq.minimize, n_trotters=m)
    a.set_preferences(algorithm=algo)
    a.seed(seed)
    a.prepare()
    return a


@pytest.mark.parametrize("N,m,algo", [(300, 32, sq.algorithm.coloring), (96, 3, sq.algorithm.coloring),
                                      (40, 6, sq.algorithm.naive), (64, 1, sq.algorithm.sa_naive)])
def test_dense_checkpoint_resumes_bit_for_bit(N, m, algo):
    W = sym_W(N, N + m)
    Gs = schedule(40)
    ref = dense(W, m, algo)
    ref.randomize_spin()
    for G in Gs:
        ref.anneal_one_step(G, BETA)
    ref.make_solution()

    a = dense(W, m, algo)
    a.randomize_spin()
    for G in Gs[:13]:
        a.anneal_one_step(G, BETA)
    state = through_file(a.get_checkpoint())
    assert state['q'].shape == (m, N) and int(state['since_refresh']) == 13 % 8
    b = dense(W, m, algo, seed=12345)  # any seed: the checkpoint carries the Philox state
    b.set_checkpoint(state)
    for G in Gs[13:]:
        a.anneal_one_step(G, BETA)
        b.anneal_one_step(G, BETA)
    a.make_solution()
    b.make_solution()
    assert np.array_equal(np.array(b.get_q()), np.array(ref.get_q()))
    assert np.array_equal(np.array(a.get_q()), np.array(ref.get_q()))  # taking a checkpoint changes nothing
    assert np.array_equal(b.get_E64(), ref.get_E64())


def test_bipartite_checkpoint_resumes_bit_for_bit():
    rng = np.random.default_rng(3)
    N0, N1, m = 48, 40, 8
    b0, b1 = rng.uniform(-1, 1, N0).astype(np.float32), rng.uniform(-1, 1, N1).astype(np.float32)
    W = rng.uniform(-1, 1, (N1, N0)).astype(np.float32)
    Gs = schedule(30)

    def make(seed=5):
        a = sq.cuda.bipartite_graph_annealer(b0, b1, W, sq.minimize, n_trotters=m)
        a.seed(seed)
        a.prepare()
        return a

    ref = make()
    ref.randomize_spin()
    for G in Gs:
        ref.anneal_one_step(G, BETA)
    ref.make_solution()
    a = make()
    a.randomize_spin()
    for G in Gs[:11]:
        a.anneal_one_step(G, BETA)
    state = through_file(a.get_checkpoint())
    b = make(seed=999)
    b.set_checkpoint(state)
    for G in Gs[11:]:
        b.anneal_one_step(G, BETA)
    b.make_solution()
    for (p0, p1), (r0, r1) in zip(b.get_q(), ref.get_q()):
        assert np.array_equal(p0, r0) and np.array_equal(p1, r1)
    assert np.array_equal(b.get_E64(), ref.get_E64())


def test_checkpoint_rejects_a_mismatched_annealer():
    W = sym_W(64, 1)
    a = dense(W, 8, sq.algorithm.coloring)
    a.randomize_spin()
    state = a.get_checkpoint()
    other = dense(W, 4, sq.algorithm.coloring)
    with pytest.raises(sq.SqaodError, match="Shape does not match"):
        other.set_checkpoint(state)
    bad = dict(state)
    bad['q'] = np.zeros_like(state['q'])
    with pytest.raises(sq.SqaodError, match="q must be -1 or"):
        a.set_checkpoint(bad)
    bad = dict(state)
    bad['since_refresh'] = np.int32(9)
    with pytest.raises(sq.SqaodError, match="refresh out of range"):
        a.set_checkpoint(bad)
