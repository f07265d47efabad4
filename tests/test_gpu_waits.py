"""Bounded device waits give up, report, and leave the GPU usable.

The one-CTA-per-trotter sweep waits on its ring neighbours' accept words and on
its own prefetcher warps; every such wait is bounded by the global timer.  Two
task flags (test hooks) make a wait run out without any fault: waits give up
after 1 ms, and trotter 0 never publishes its accept words, so its neighbours
(and, in turn, theirs) stop at their first wait on it.  The kernel then ends
with status 1, the annealer raises at its next synchronising call, and a normal
anneal on the same device replays against FP64 as usual.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHORT_WAITS, WITHHOLD_TROTTER0 = 16, 32


def _sym(rng, N):
    W = rng.uniform(-1, 1, (N, N))
    return (np.triu(W) + np.triu(W, 1).T).astype(np.float32)


@pytest.mark.parametrize("N,m", [(1024, 16), (256, 3)])
def test_sweep_wait_gives_up_and_gpu_stays_usable(orc, N, m):
    import sqaod_gb300 as sq
    rng = np.random.default_rng(N + m)
    W = _sym(rng, N)
    G = np.array([5.0 * 0.9 ** k for k in range(8)], np.float32)
    a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm="coloring")
    a.set_kernel(2 | SHORT_WAITS | WITHHOLD_TROTTER0)
    a.seed(3)
    a.prepare()
    a.randomize_spin()
    t0 = time.time()
    a.anneal(G, 20.0)
    with pytest.raises(RuntimeError, match="timed out"):
        a.get_q()
    elapsed = time.time() - t0
    print("N=%d m=%d: the sweep gave up after %.3f s" % (N, m, elapsed))
    assert elapsed < 3.0  # 1 ms waits, not the 4 s default

    # the same annealer and device then anneal normally, replayed against FP64
    a.set_kernel(2)
    a.prepare()
    a.randomize_spin()
    q = np.array(a.get_q())
    h, J, c = a.get_hamiltonian()
    a.set_trace(True)
    _, step0 = a.get_rng_state()
    a.anneal(G, 20.0)
    trace = a.get_trace((N * m + 31) // 32 * len(G))
    q_host, st = orc.dg_replay_steps(h, J, m, orc.ALGO_COLORING, 3, step0, G, 20.0, q, trace, 1e-6)
    assert np.array_equal(np.array(a.get_q()), q_host)
    assert st["n_mismatch"] == st["n_mismatch_small"], st


def test_short_waits_alone_do_not_fire(orc):
    """With 1 ms waits but every trotter publishing, no wait comes near its
    limit: the anneal completes and replays."""
    import sqaod_gb300 as sq
    rng = np.random.default_rng(5)
    N, m = 512, 8
    W = _sym(rng, N)
    G = np.array([5.0 * 0.9 ** k for k in range(8)], np.float32)
    a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm="coloring")
    a.set_kernel(2 | SHORT_WAITS)
    a.seed(4)
    a.prepare()
    a.randomize_spin()
    q = np.array(a.get_q())
    h, J, c = a.get_hamiltonian()
    a.set_trace(True)
    _, step0 = a.get_rng_state()
    a.anneal(G, 20.0)
    trace = a.get_trace((N * m + 31) // 32 * len(G))
    q_host, st = orc.dg_replay_steps(h, J, m, orc.ALGO_COLORING, 4, step0, G, 20.0, q, trace, 1e-6)
    assert np.array_equal(np.array(a.get_q()), q_host)
    assert st["n_mismatch"] == st["n_mismatch_small"], st


def test_kernel_selector_rejects_unknown_flags():
    import sqaod_gb300 as sq
    a = sq.cuda.dense_graph_annealer(_sym(np.random.default_rng(0), 64), n_trotters=4)
    for bad in (3, 64, 2 | 128, -1):
        with pytest.raises(RuntimeError, match="kernel selector"):
            a.set_kernel(bad)
