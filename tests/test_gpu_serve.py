"""Request server: dense and bipartite requests of mixed size, trotter count and
schedule length, admitted under a tight memory budget and a small slot limit
(so requests queue, finish at different ticks and slots are compacted), each
end bit-identical to annealing the same request alone with the single-instance
annealer."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _schedule(n, g0=5.0):
    return (g0 * 0.93 ** np.arange(n)).astype(np.float32), np.linspace(10.0, 40.0, n).astype(np.float32)


def _sym(rng, N):
    W = rng.uniform(-1, 1, (N, N))
    return (np.triu(W) + np.triu(W, 1).T).astype(np.float32)


# (kind, sizes, m, steps, optimize)
SPECS = [
    ("d", 40, 8, 12, "min"),
    ("d", 96, 1, 20, "min"),
    ("b", (24, 40), 4, 9, "min"),
    ("d", 200, 16, 17, "max"),
    ("d", 1024, 64, 10, "min"),  # beyond shared-memory staging: one CTA per trotter
    ("b", (64, 32), 1, 15, "min"),
    ("d", 130, 2, 25, "min"),
    ("b", (48, 48), 8, 11, "max"),
    ("d", 64, 32, 3, "min"),
    ("d", 1023, 16, 9, "min"),  # one CTA per trotter, row stride padded to 1024
    ("b", (1024, 512), 16, 7, "min"),  # per-instance bipartite kernels
]


def _alone(sq, spec, data, seed):
    kind, sizes, m, steps, opt = spec
    G, beta = _schedule(steps)
    o = sq.maximize if opt == "max" else sq.minimize
    if kind == "d":
        a = sq.cuda.dense_graph_annealer(data, o, n_trotters=m, algorithm="sa_naive" if m == 1 else "coloring")
    else:
        b0, b1, W = data
        a = sq.cuda.bipartite_graph_annealer(b0, b1, W, o, n_trotters=m,
                                             algorithm="sa_coloring" if m == 1 else "coloring")
    a.seed(seed)
    a.prepare()
    a.randomize_spin()
    a.anneal(G, beta)
    return a.get_E64(), a.get_q()


def test_server_requests_match_alone():
    import sqaod_gb300 as sq
    from sqaod_gb300.serve import DONE, AnnealServer
    rng = np.random.default_rng(11)
    data = []
    for kind, sizes, m, steps, opt in SPECS:
        if kind == "d":
            data.append(_sym(rng, sizes))
        else:
            N0, N1 = sizes
            data.append((rng.uniform(-1, 1, N0).astype(np.float32), rng.uniform(-1, 1, N1).astype(np.float32),
                         rng.uniform(-1, 1, (N1, N0)).astype(np.float32)))
    # the N=1024 request (about 5 MB) waits until enough of the others finish; one
    # large instance at a time
    srv = AnnealServer(budget_bytes=6 << 20, max_slots=3)
    srv.set_large_limit(1)
    ids = []
    for i, (spec, d) in enumerate(zip(SPECS, data)):
        kind, sizes, m, steps, opt = spec
        G, beta = _schedule(steps)
        o = sq.maximize if opt == "max" else sq.minimize
        if kind == "d":
            ids.append(srv.submit_dense(d, m, G, beta, o, seed=1000 + i))
        else:
            ids.append(srv.submit_bipartite(d[0], d[1], d[2], m, G, beta, o, seed=1000 + i))
    ticks = srv.run(max_ticks=500)
    assert ticks < 500
    st = srv.stats()
    assert st["queued"] == 0 and st["active"] == 0 and st["done"] == len(SPECS)
    assert st["bytes_in_use"] == 0
    # queueing made the run longer than the longest request (8 steps per tick)
    assert ticks > -(-max(s[3] for s in SPECS) // 8)
    for i, (spec, d, rid) in enumerate(zip(SPECS, data, ids)):
        assert srv.state(rid) == DONE
        E, q = srv.result(rid)
        E1, q1 = _alone(sq, spec, d, 1000 + i)
        assert np.array_equal(E, E1), (i, E, E1)
        if spec[0] == "d":
            assert np.array_equal(q, np.array(q1)), i
        else:
            assert np.array_equal(q[0], np.array([p[0] for p in q1])), i
            assert np.array_equal(q[1], np.array([p[1] for p in q1])), i


def test_server_packs_large_dense_requests():
    """Large dense requests of different sizes and lengths step together in
    packed cooperative launches; each still ends bit-identical to annealing it alone."""
    import sqaod_gb300 as sq
    from sqaod_gb300.serve import AnnealServer
    specs = [("d", 1024, 64, 17, "min"), ("d", 700, 32, 9, "max"), ("d", 1500, 16, 12, "min"),
             ("d", 257, 128, 20, "min"), ("d", 1024, 40, 8, "min")]
    rng = np.random.default_rng(23)
    data = [_sym(rng, sp[1]) for sp in specs]
    srv = AnnealServer(budget_bytes=1 << 30, max_slots=8)
    srv.set_large_limit(8)
    ids = []
    for i, (spec, d) in enumerate(zip(specs, data)):
        G, beta = _schedule(spec[3])
        ids.append(srv.submit_dense(d, spec[2], G, beta, sq.maximize if spec[4] == "max" else sq.minimize,
                                    seed=2000 + i))
    assert srv.run(max_ticks=100) < 100
    for i, (spec, d, rid) in enumerate(zip(specs, data, ids)):
        E, q = srv.result(rid)
        E1, q1 = _alone(sq, spec, d, 2000 + i)
        assert np.array_equal(E, E1), (i, E, E1)
        assert np.array_equal(q, np.array(q1)), i


def test_server_rejects_oversized_request():
    import sqaod_gb300 as sq
    from sqaod_gb300._lib import SqaodError
    from sqaod_gb300.serve import AnnealServer
    srv = AnnealServer(budget_bytes=1 << 20)
    G, beta = _schedule(4)
    with pytest.raises(SqaodError, match="exceeds the device-memory budget"):
        srv.submit_dense(_sym(np.random.default_rng(0), 1024), 4, G, beta, sq.minimize)
    assert srv.stats()["queued"] == 0
