"""Multi-GPU / multi-process sharding of the Similarity path.

Pairs are independent, so N workers (one process per GPU) take disjoint,
contiguous ranges of KINC's 32,768-pair work blocks and never exchange data
while computing.  Because the ranges are contiguous in pair order, each
worker's CCM/CMX items are already sorted and the global item lists are the
concatenation of the per-worker lists in rank order -- the only
communication is that final gather (over files, sockets or a
torch.distributed gather of host objects), never a collective on the GPU data
path.  rand() positions stay exact on every worker because the GPU derives
each block's position from its first pair.
"""
from dataclasses import dataclass

WORK_BLOCK_SIZE = 32768


@dataclass
class Shard:
    rank: int
    start: int          # first pair
    size: int           # pairs

    @property
    def end(self):
        return self.start + self.size


def total_pairs(genes):
    return genes * (genes - 1) // 2


def shard_pairs(genes, world, rank, block=WORK_BLOCK_SIZE):
    """Contiguous range of whole work blocks for `rank` of `world` (balanced by block count)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    total = total_pairs(genes)
    nblocks = (total + block - 1) // block
    b0 = nblocks * rank // world
    b1 = nblocks * (rank + 1) // world
    start = min(b0 * block, total)
    end = min(b1 * block, total)
    return Shard(rank, start, end - start)


def block_costs(gem, min_expr=float("-inf"), block=WORK_BLOCK_SIZE):
    """Estimated cost of every work block: the sum over its pairs of n_x * n_y / S, with n_g the
    gene's usable samples -- the expected pairwise usable count when missing values are
    independent, to which every per-pair pass (fetch, EM and Lloyd sweeps, correlations) is
    proportional.  O(genes + blocks): each row of pairs spans at most two blocks while
    genes < block, and is summed from a prefix over n_y."""
    import numpy as np
    gem = np.asarray(gem)
    G, S = gem.shape
    usable = ~np.isnan(gem) & ~(gem < min_expr)
    n = usable.sum(axis=1).astype(np.float64)
    prefix = np.concatenate([[0.0], np.cumsum(n)])
    total = total_pairs(G)
    nblocks = (total + block - 1) // block
    costs = np.zeros(nblocks, np.float64)
    for x in range(1, G):
        p0 = x * (x - 1) // 2          # pairs (x, 0) .. (x, x-1)
        y = 0
        while y < x:
            b = (p0 + y) // block
            y_end = min(x, (b + 1) * block - p0)
            costs[b] += n[x] * (prefix[y_end] - prefix[y]) / max(S, 1)
            y = y_end
    return costs


def shard_pairs_by_cost(costs, genes, world, rank, block=WORK_BLOCK_SIZE):
    """Contiguous range of whole work blocks for `rank` of `world`, cut where the running sum of
    the blocks' estimated costs crosses rank/world and (rank+1)/world of the total."""
    import numpy as np
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    total = total_pairs(genes)
    c = np.concatenate([[0.0], np.cumsum(np.asarray(costs, np.float64))])
    whole = c[-1]
    if whole <= 0:
        return shard_pairs(genes, world, rank, block)

    def cut(r):
        if r <= 0:
            return 0
        if r >= world:
            return len(costs)
        return int(np.searchsorted(c, whole * r / world, side="left"))

    b0, b1 = cut(rank), cut(rank + 1)
    start = min(b0 * block, total)
    end = min(b1 * block, total)
    return Shard(rank, start, max(end - start, 0))


def merge_items(per_rank):
    """Concatenate per-rank item lists (each a dict of equal-length sequences) in rank order,
    checking that the pair order is strictly increasing across the seams."""
    keys = None
    out = {}
    last = -1
    for items in per_rank:
        if keys is None:
            keys = list(items.keys())
            out = {k: [] for k in keys}
        n = len(items["x"])
        if n:
            first = int(items["x"][0]) * (int(items["x"][0]) - 1) // 2 + int(items["y"][0])
            if first * 64 + int(items["c"][0]) <= last:
                raise ValueError("shards overlap or are out of order")
            lx, ly, lc = int(items["x"][-1]), int(items["y"][-1]), int(items["c"][-1])
            last = (lx * (lx - 1) // 2 + ly) * 64 + lc
        for k in keys:
            out[k].extend(list(items[k]))
    return out


def shard_blocks(gem, world, rank, by_cost=False, min_expr=float("-inf")):
    """The native partition (include/kinc_sim.h: kinc_shard_blocks): (first_block, nblocks) of
    KINC's 32,768-pair work blocks for `rank`, by block count or by estimated cost -- the same
    cut as shard_pairs / shard_pairs_by_cost at that block size."""
    import ctypes

    import numpy as np

    from . import _native
    gem = np.ascontiguousarray(gem, np.float32)
    first, n = ctypes.c_int64(), ctypes.c_int64()
    rc = _native.load().kinc_shard_blocks(gem.ctypes.data_as(ctypes.c_void_p), gem.shape[0], gem.shape[1],
                                          float(min_expr), int(world), int(rank), int(bool(by_cost)),
                                          ctypes.byref(first), ctypes.byref(n))
    if rc != _native.OK:
        raise ValueError(f"rank {rank} outside world of {world}, or a matrix of fewer than 2 genes")
    return first.value, n.value
