"""Batched annealing of uneven instances: each instance ends bit-identical to
annealing it alone with the single-instance solver and the same seed, with and
without CUDA-graph replay, whatever launch configuration the autotuner picks."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _schedule(n):
    G, g = [], 5.0
    for _ in range(n):
        G.append(g)
        g *= 0.97
    return np.array(G, np.float32)


def _problems(k, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    # small instances (one CTA each in the persistent launch) and, last, instances
    # too large to stage (packed one-CTA-per-trotter launches; N = 1030 pads its rows)
    shapes = [(int(rng.choice([40, 64, 96, 130, 200, 256])), int(rng.choice([1, 2, 8, 16, 32]))) for _ in range(k)]
    shapes += [(600, 24), (1030, 16), (300, 64)]
    for i, (N, m) in enumerate(shapes):
        W = rng.uniform(-1, 1, (N, N))
        W = (np.triu(W) + np.triu(W, 1).T).astype(np.float32)
        out.append((W, m, 100 + i))
    return out


@pytest.mark.parametrize("use_graph,min_n", [(True, None), (False, None), (True, 0), (False, 64), (True, 512)])
def test_batch_equals_single(use_graph, min_n):
    import sqaod_gb300 as sq
    from sqaod_gb300.batch import DenseBatchAnnealer
    probs = _problems(12)
    G = _schedule(20)
    b = DenseBatchAnnealer()
    for W, m, seed in probs:
        b.add(W, m, sq.minimize, seed)
    b.set_schedule(G, 30.0)
    if min_n is not None:
        b.set_multicta_min_n(min_n)
    b.prepare()
    # instances of at least min_n spins (default 1024) and m >= 2 take the packed launches
    limit = 1024 if min_n is None else min_n
    expect = sum(1 for W, m, _ in probs if limit > 0 and W.shape[0] >= limit and m >= 2)
    assert b.multicta_count() == expect
    b.autotune(2)
    # uneven calls: chunks must still end at the field refreshes
    b.anneal(5, use_graph=use_graph)
    b.anneal(len(G) - 5, use_graph=use_graph)
    assert b.info()["position"] == len(G)
    for i, (W, m, seed) in enumerate(probs):
        # one trotter runs simulated annealing in the batch
        a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm="sa_naive" if m == 1 else "coloring")
        a.set_kernel(1)
        a.seed(seed)
        a.prepare()
        a.randomize_spin()
        a.anneal(G, 30.0)
        assert np.array_equal(np.array(a.get_q()), b.get_q(i)), i
        assert np.array_equal(a.get_E64(), b.get_E64(i)), i


def test_batch_routing_autotune_keeps_results():
    """autotune_routing times each candidate size limit from a fresh prepare and
    prepares again with the fastest: it returns one of the candidates, the
    packed-instance count follows it, and every instance still ends as alone."""
    import sqaod_gb300 as sq
    from sqaod_gb300.batch import DenseBatchAnnealer
    probs = _problems(10, seed=3)
    G = _schedule(12)
    b = DenseBatchAnnealer()
    for W, m, seed in probs:
        b.add(W, m, sq.minimize, seed)
    b.set_schedule(G, 30.0)
    b.prepare()
    cands = (0, 256, 1024)
    chosen = b.autotune_routing(4, cands)
    assert chosen in cands
    expect = sum(1 for W, m, _ in probs if chosen > 0 and W.shape[0] >= chosen and m >= 2)
    assert b.multicta_count() == expect
    assert b.info()["position"] == 0
    b.anneal(len(G))
    for i, (W, m, seed) in enumerate(probs):
        a = sq.cuda.dense_graph_annealer(W, n_trotters=m, algorithm="sa_naive" if m == 1 else "coloring")
        a.seed(seed)
        a.prepare()
        a.randomize_spin()
        a.anneal(G, 30.0)
        assert np.array_equal(np.array(a.get_q()), b.get_q(i)), i
        assert np.array_equal(a.get_E64(), b.get_E64(i)), i


def test_field_refresh_batch_equals_single_refresh():
    """sq103_dense_field_refresh_batch (one launch over every job's tiles) gives
    each job the fields of its own sq103_dense_field_refresh, bit for bit: ragged
    N and m, more than 64 trotters, padded rows (the padding holds NaN, so a read
    past N would show)."""
    import ctypes
    torch = pytest.importorskip("torch")
    from sqaod_gb300 import _lib
    L = _lib.lib()

    class FieldJob(ctypes.Structure):
        _fields_ = [("J", ctypes.c_void_p), ("q", ctypes.c_void_p), ("F", ctypes.c_void_p),
                    ("N", ctypes.c_int), ("m", ctypes.c_int), ("ldJ", ctypes.c_int), ("tile0", ctypes.c_int)]

    dev = torch.device("cuda", 0)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(7)
    shapes = [(40, 3), (64, 64), (100, 65), (130, 16), (37, 128), (1, 1), (200, 8), (513, 33)]
    jobs, tile_job, keep, singles = [], [], [], []
    for j, (N, m) in enumerate(shapes):
        ldJ = (N + 3) & ~3
        Jh = np.full((N, ldJ), np.nan, np.float32)
        Jh[:, :N] = rng.uniform(-1, 1, (N, N)).astype(np.float32)
        qh = rng.choice(np.array([-1, 1], np.int8), (m, N))
        dJ = torch.from_numpy(Jh).to(dev)
        dq = torch.from_numpy(qh).to(dev)
        Fb = torch.full((m, N), -7.0, dtype=torch.float32, device=dev)
        Fs = torch.empty((m, N), dtype=torch.float32, device=dev)
        assert L.sq103_dense_field_refresh(ctypes.c_void_p(dJ.data_ptr()), ldJ, ctypes.c_void_p(dq.data_ptr()),
                                           ctypes.c_void_p(Fs.data_ptr()), N, m, sp) == 0
        jobs.append(FieldJob(dJ.data_ptr(), dq.data_ptr(), Fb.data_ptr(), N, m, ldJ, len(tile_job)))
        tile_job += [j] * (((N + 63) // 64) * ((m + 63) // 64))
        keep += [dJ, dq]
        singles.append((Fs, Fb))
    arr = (FieldJob * len(jobs))(*jobs)
    dJobs = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)
    dTiles = torch.tensor(tile_job, dtype=torch.int32, device=dev)
    assert L.sq103_dense_field_refresh_batch(ctypes.c_void_p(dJobs.data_ptr()), ctypes.c_void_p(dTiles.data_ptr()),
                                             len(tile_job), sp) == 0
    torch.cuda.synchronize()
    for (N, m), (Fs, Fb) in zip(shapes, singles):
        assert torch.equal(Fs.view(torch.int32), Fb.view(torch.int32)), (N, m)
        assert torch.isfinite(Fb).all(), (N, m)
    assert L.sq103_dense_field_refresh_batch(None, None, 0, sp) == 0
    assert L.sq103_dense_field_refresh_batch(None, None, 3, sp) != 0
