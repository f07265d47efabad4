"""Multi-GPU runs: state-range shards for brute-force search, replicas for annealing.

Brute-force search shards by state range.  Rank r of a group of W searches
the contiguous packed states [b_r, b_{r+1}) on its own GPU
(DenseGraphBFSearcher.search_subrange); one all_gather of every rank's
(FP64 minimum, minimisers) follows, and the host merge gives exactly what one
searcher over the whole range gives: the global minimum and its minimisers in
ascending packed order, the first `tile_size` of them (the tie and cap rules
of sqaodc/cpu/CPUDenseGraphBFSearcher.cpp:104-131).  There is no collective on
the data path.

Annealing does not shard: trotters are ring-coupled and every accepted flip
touches a whole field row.  Multi-GPU annealing runs independent replicas;
replica_throughput() forms the whole-job rate from the slowest rank.

Each rank selects its GPU before calling in (torch.cuda.set_device(local_rank)).
No counterpart in the reference.
"""
import numpy as np

from . import common


def shard_range(n_states, rank, world):
    """[begin, end) of rank's contiguous share of n_states (sizes differ by at most one)."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank %d outside a group of %d" % (rank, world))
    q, r = divmod(int(n_states), world)
    b = rank * q + min(rank, r)
    return b, b + q + (1 if rank < r else 0)


def merge_shards(results, cap):
    """Merges per-rank results, given in ascending range order.  Each is (E, xs):
    E the shard's minimum in the minimisation direction (inf when the shard holds
    no state) and xs its minimisers in ascending packed order.  Returns the
    global (Emin, first `cap` minimisers ascending)."""
    found = [E for E, xs in results if len(xs)]
    if not found:
        return float("inf"), np.zeros(0, np.uint64)
    Emin = min(found)
    out = []
    for E, xs in results:
        if E != Emin:
            continue
        for x in xs:
            if len(out) >= cap:
                break
            out.append(int(x))
    return Emin, np.array(out, np.uint64)


def pack_bits(x):
    """Packed value of a bit row, variable i at bit N-1-i (sqaodc/common/Common.cpp:79-93)."""
    v = 0
    for b in x:
        v = (v << 1) | int(b)
    return v


def gpu_shard_search(W, optimize, begin, end, tile_size):
    """One rank's shard on the current GPU: (E in the minimisation direction, minimisers)."""
    from .cuda import dense_graph_bf_searcher
    s = dense_graph_bf_searcher(W, optimize, tile_size=tile_size)
    s.prepare()
    s.search_subrange(begin, end)
    E = s.get_E64()
    if not np.isfinite(E) or abs(E) >= np.finfo(np.float64).max:
        return float("inf"), []
    s.make_solution()
    xs = [pack_bits(x) for x in s.get_x()]
    return (-E if common.optimize_flag(optimize) else E), xs


def dense_bf_search(W, optimize=common.minimize, tile_size=1 << 18, group=None, shard_search=None):
    """Brute-force search of a dense QUBO over the ranks of `group` (a
    torch.distributed process group; None = the default one).  Every rank
    returns the same (E, minimisers): E in the user's direction (the maximum
    for maximize), the minimisers as packed values in ascending order.
    shard_search(W, optimize, begin, end, cap) -> (E_min_direction, xs) searches
    one shard (default: this rank's GPU)."""
    import torch.distributed as dist
    W = np.asarray(W)
    common.check_square(W)
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    begin, end = shard_range(1 << W.shape[0], rank, world)
    E, xs = (shard_search or gpu_shard_search)(W, optimize, begin, end, tile_size)
    gathered = [None] * world
    dist.all_gather_object(gathered, (float(E), [int(v) for v in xs]), group=group)
    Emin, out = merge_shards(gathered, tile_size)
    return (-Emin if common.optimize_flag(optimize) else Emin), out


def replica_throughput(local_ms, units_per_rank, group=None, device=None):
    """Whole-job rate of independent replicas: the units all ranks processed
    over the slowest rank's time.  Returns (units per second, max ms)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
        world = dist.get_world_size(group)
    else:
        world = 1
    t_max = float(t.item())
    return float(units_per_rank) * world / (t_max / 1e3), t_max
