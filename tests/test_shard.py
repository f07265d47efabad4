"""Multi-GPU host logic on CPU: state-range shards of the brute-force search
and their merge (checked against one search of the whole range by the oracle),
and the replica throughput over ranks -- as two gloo ranks on this host."""
import os
import socket

import numpy as np
import pytest

from sqaod_gb300 import common, shard


def _int_sym(rng, N, lo=-4, hi=4):
    U = np.triu(rng.integers(lo, hi + 1, (N, N)))
    return (U + np.triu(U, 1).T).astype(np.float32)


def _oracle_shard(W, optimize, begin, end, cap):
    """One shard searched by the oracle, in the shard_search convention."""
    from oracle import oracle_ctypes as orc
    if begin >= end:
        return float("inf"), []
    om = common.optimize_flag(optimize)
    E, xs = orc.dg_bf_search_range(W, om, begin, end, cap)
    return (-float(E) if om else float(E)), sorted(int(v) for v in xs)


def test_shard_range_partitions():
    for n in (0, 1, 7, 16, 1 << 20, (1 << 20) + 3):
        for world in (1, 2, 3, 8):
            spans = [shard.shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(spans[r][1] == spans[r + 1][0] for r in range(world - 1))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.shard_range(8, 2, 2)


@pytest.mark.parametrize("opt", ["min", "max"])
@pytest.mark.parametrize("world", [2, 3, 5])
def test_merged_shards_equal_whole_range(orc, opt, world):
    import sqaod_gb300 as sq
    optimize = sq.maximize if opt == "max" else sq.minimize
    W = _int_sym(np.random.default_rng(world), 11)
    cap = 1 << 11
    parts = [_oracle_shard(W, optimize, *shard.shard_range(1 << 11, r, world), cap) for r in range(world)]
    E, xs = shard.merge_shards(parts, cap)
    E_all, xs_all = orc.dg_bf_search_range(W, 1 if opt == "max" else 0, 0, 1 << 11, cap)
    assert (-E if opt == "max" else E) == E_all
    assert xs.tolist() == sorted(int(v) for v in xs_all)


def test_merge_keeps_the_first_cap_minimisers(orc):
    # W = 0: every state is a minimiser; the first `cap` in ascending order survive
    W = np.zeros((10, 10), np.float32)
    parts = [_oracle_shard(W, 0, *shard.shard_range(1 << 10, r, 4), 40) for r in range(4)]
    E, xs = shard.merge_shards(parts, 40)
    assert E == 0.0 and xs.tolist() == list(range(40))
    assert shard.merge_shards([(float("inf"), []), (float("inf"), [])], 8)[1].size == 0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, W, opt, cap, out):
    import torch.distributed as dist
    import sqaod_gb300 as sq
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        optimize = sq.maximize if opt == "max" else sq.minimize
        E, xs = shard.dense_bf_search(W, optimize, tile_size=cap, shard_search=_oracle_shard)
        rate, t_max = shard.replica_throughput(10.0 * (rank + 1), 1000.0)
        out.put((rank, E, xs.tolist(), rate, t_max))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("opt", ["min", "max"])
def test_two_gloo_ranks(orc, opt):
    import torch.multiprocessing as mp
    W = _int_sym(np.random.default_rng(7), 12)
    cap = 64
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, W, opt, cap, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = [out.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    E_all, xs_all = orc.dg_bf_search_range(W, 1 if opt == "max" else 0, 0, 1 << 12, cap)
    for rank, E, xs, rate, t_max in res:
        assert E == E_all and xs == sorted(int(v) for v in xs_all)[:cap]
        # replicas: 2 x 1000 units over the slower rank's 20 ms
        assert t_max == 20.0 and rate == pytest.approx(2 * 1000.0 / 0.020)
