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
    # the N=1024 request (about 14 MB with its digit planes) waits until enough of the others finish; one
    # large instance at a time
    srv = AnnealServer(budget_bytes=16 << 20, max_slots=3)
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


def test_server_large_bipartite_requests_side_by_side():
    """Large bipartite requests (m N0 N1 > 2^22, the per-instance kernels) of
    different shapes and lengths step side by side on the server's side streams,
    beside large and small dense requests whose fields refresh in the same
    ticks; each ends bit-identical to annealing it alone."""
    import sqaod_gb300 as sq
    from sqaod_gb300.serve import AnnealServer
    specs = [("b", (512, 512), 32, 17, "min"), ("b", (300, 400), 64, 9, "max"), ("b", (256, 1024), 24, 12, "min"),
             ("b", (2048, 1024), 8, 10, "min"), ("b", (640, 200), 40, 20, "max"),
             ("b", (2048, 2048), 256, 8, "min"),  # half-step fields on the tensor cores
             ("d", 1500, 16, 12, "min"),
             ("d", 1024, 8, 16, "min"), ("d", 300, 16, 11, "min"), ("d", 80, 4, 9, "max")]
    rng = np.random.default_rng(31)
    data = []
    for kind, sizes, m, steps, opt in specs:
        if kind == "d":
            data.append(_sym(rng, sizes))
        else:
            N0, N1 = sizes
            data.append((rng.uniform(-1, 1, N0).astype(np.float32), rng.uniform(-1, 1, N1).astype(np.float32),
                         rng.uniform(-1, 1, (N1, N0)).astype(np.float32)))
    srv = AnnealServer(budget_bytes=1 << 30, max_slots=8)
    srv.set_large_limit(16)
    ids = []
    for i, (spec, d) in enumerate(zip(specs, data)):
        kind, sizes, m, steps, opt = spec
        G, beta = _schedule(steps)
        o = sq.maximize if opt == "max" else sq.minimize
        if kind == "d":
            ids.append(srv.submit_dense(d, m, G, beta, o, seed=3100 + i))
        else:
            ids.append(srv.submit_bipartite(d[0], d[1], d[2], m, G, beta, o, seed=3100 + i))
    srv.tick()
    assert srv.stats()["active"] == len(specs)  # all admitted together
    assert srv.run(max_ticks=100) < 100
    for i, (spec, d, rid) in enumerate(zip(specs, data, ids)):
        E, q = srv.result(rid)
        E1, q1 = _alone(sq, spec, d, 3100 + i)
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


def test_server_packs_more_than_eight_requests():
    """Twelve large small-m dense requests fit one packed cooperative launch
    (up to 16 instances per launch); each still ends bit-identical to annealing
    it alone."""
    import sqaod_gb300 as sq
    from sqaod_gb300.serve import AnnealServer
    specs = [("d", 900 + 8 * k, 24, 10 + k % 3, "min") for k in range(12)]
    rng = np.random.default_rng(29)
    data = [_sym(rng, sp[1]) for sp in specs]
    srv = AnnealServer(budget_bytes=1 << 30, max_slots=4)
    srv.set_large_limit(16)
    ids = []
    for i, (spec, d) in enumerate(zip(specs, data)):
        G, beta = _schedule(spec[3])
        ids.append(srv.submit_dense(d, spec[2], G, beta, sq.minimize, seed=2500 + i))
    srv.tick()
    assert srv.stats()["active"] == 12  # all admitted together: one pack of twelve
    assert srv.run(max_ticks=100) < 100
    for i, (spec, d, rid) in enumerate(zip(specs, data, ids)):
        E, q = srv.result(rid)
        E1, q1 = _alone(sq, spec, d, 2500 + i)
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


def test_server_admits_arrivals_between_ticks():
    """Requests submitted while others are on the GPU (between tick() calls,
    under a budget and slot limit that make some wait) start as memory and slots
    free up; each ends bit-identical to annealing it alone."""
    import sqaod_gb300 as sq
    from sqaod_gb300.serve import AnnealServer
    rng = np.random.default_rng(31)
    waves = [[("d", 300, 16, 20, "min"), ("b", (64, 80), 8, 14, "min")],
             [("d", 1024, 32, 17, "min"), ("d", 50, 1, 9, "max")],
             [("b", (40, 24), 1, 12, "min"), ("d", 180, 8, 30, "min"), ("d", 700, 16, 10, "min")]]
    srv = AnnealServer(budget_bytes=16 << 20, max_slots=2)
    srv.set_large_limit(1)
    subs = []
    for w, wave in enumerate(waves):
        for spec in wave:
            kind, sizes, m, steps, opt = spec
            G, beta = _schedule(steps)
            o = sq.maximize if opt == "max" else sq.minimize
            seed = 3000 + len(subs)
            if kind == "d":
                d = _sym(rng, sizes)
                rid = srv.submit_dense(d, m, G, beta, o, seed=seed)
            else:
                N0, N1 = sizes
                d = (rng.uniform(-1, 1, N0).astype(np.float32), rng.uniform(-1, 1, N1).astype(np.float32),
                     rng.uniform(-1, 1, (N1, N0)).astype(np.float32))
                rid = srv.submit_bipartite(d[0], d[1], d[2], m, G, beta, o, seed=seed)
            subs.append((spec, d, seed, rid))
        if w < len(waves) - 1:
            srv.tick()
            s = srv.stats()
            assert s["active"] > 0  # the next wave arrives while these are on the GPU
    assert srv.run(max_ticks=200) < 200
    for spec, d, seed, rid in subs:
        E, q = srv.result(rid)
        E1, q1 = _alone(sq, spec, d, seed)
        assert np.array_equal(E, E1), (spec, E, E1)
        if spec[0] == "d":
            assert np.array_equal(q, np.array(q1)), spec
        else:
            assert np.array_equal(q[0], np.array([p[0] for p in q1])), spec
            assert np.array_equal(q[1], np.array([p[1] for p in q1])), spec


def test_server_status_is_per_request():
    """A dense request whose status word reports a given-up device wait (set
    from the host, as the sweep would) fails alone: the others, and requests
    submitted after it, still complete and match their single-instance runs."""
    import sqaod_gb300 as sq
    from sqaod_gb300.serve import AnnealServer
    rng = np.random.default_rng(41)
    specs = [("d", 64, 4, 16, "min"), ("d", 1024, 16, 16, "min"), ("d", 96, 8, 16, "min")]
    data = [_sym(rng, sp[1]) for sp in specs]
    srv = AnnealServer(budget_bytes=1 << 30)
    ids = []
    for i, (spec, d) in enumerate(zip(specs, data)):
        G, beta = _schedule(spec[3])
        ids.append(srv.submit_dense(d, spec[2], G, beta, sq.minimize, seed=4000 + i))
    srv.tick()
    srv.inject_status(ids[1], 1)  # the large (one-CTA-per-trotter) request
    assert srv.run(max_ticks=50) < 50
    with pytest.raises(RuntimeError, match="bounded device wait"):
        srv.result(ids[1])
    assert srv.state_or_none(ids[1]) is None  # released all the same
    for i in (0, 2):
        E, q = srv.result(ids[i])
        E1, q1 = _alone(sq, specs[i], data[i], 4000 + i)
        assert np.array_equal(E, E1) and np.array_equal(q, np.array(q1))
    G, beta = _schedule(16)
    late = srv.submit_dense(data[1], 16, G, beta, sq.minimize, seed=4001)
    assert srv.run(max_ticks=50) < 50
    E, q = srv.result(late)
    E1, q1 = _alone(sq, specs[1], data[1], 4001)
    assert np.array_equal(E, E1) and np.array_equal(q, np.array(q1))


def _search_alone(sq, W, opt, tile):
    s = sq.cuda.dense_graph_bf_searcher(W, opt, tile_size=tile)
    s.search()
    return s.get_E64(), np.array(s.get_x())


def test_server_searches_match_alone():
    """Brute-force searches served beside anneals (some submitted between
    ticks, one larger than a tick's 2^30 states): each gives the exact minimum
    and the same minimisers, in the same order, as the single-instance search;
    the anneals still match theirs."""
    import sqaod_gb300 as sq
    from sqaod_gb300.serve import DONE, AnnealServer
    rng = np.random.default_rng(51)

    def int_sym(N, lo=-3, hi=4):
        U = np.triu(rng.integers(lo, hi, (N, N)))
        return (U + np.triu(U, 1).T).astype(np.float32)

    # (W, optimize, tile_size): integer couplings give ties, so the lists have many entries
    searches = [(int_sym(12), sq.minimize, 1 << 18), (int_sym(20, 0, 2), sq.maximize, 1 << 18),
                (int_sym(16, -1, 2), sq.minimize, 5), (_sym(rng, 24), sq.minimize, 1 << 18),
                (int_sym(31), sq.minimize, 1 << 18)]
    srv = AnnealServer(budget_bytes=1 << 30)
    G, beta = _schedule(16)
    spec_a = ("d", 256, 8, 16, "min")
    Wa = _sym(rng, 256)
    ida = srv.submit_dense(Wa, 8, G, beta, sq.minimize, seed=5000)
    ids = [srv.submit_search(W, o, tile_size=t) for W, o, t in searches[:2]]
    srv.tick()
    ids += [srv.submit_search(W, o, tile_size=t) for W, o, t in searches[2:]]
    assert srv.run(max_ticks=100) < 100
    for (W, o, t), rid in zip(searches, ids):
        assert srv.state(rid) == DONE
        E, x = srv.result(rid)
        E1, x1 = _search_alone(sq, W, o, t)
        assert E == E1, (E, E1)
        assert np.array_equal(x, x1), (x.shape, x1.shape)
        assert len(x) <= t and len(x) >= 1
    E, q = srv.result(ida)
    E1, q1 = _alone(sq, spec_a, Wa, 5000)
    assert np.array_equal(E, E1) and np.array_equal(q, np.array(q1))


def test_server_rejects_bad_search():
    from sqaod_gb300._lib import SqaodError
    from sqaod_gb300.serve import AnnealServer
    srv = AnnealServer(budget_bytes=1 << 30)
    with pytest.raises(SqaodError, match="0 < N < 64"):
        srv.submit_search(np.zeros((64, 64), np.float32))
    W = np.arange(9, dtype=np.float32).reshape(3, 3)
    with pytest.raises(RuntimeError, match="not triangular nor symmetric"):
        srv.submit_search(W + W.T + np.array([[0, 1, 0], [0, 0, 0], [0, 0, 0]], np.float32))
    assert srv.stats()["queued"] == 0
