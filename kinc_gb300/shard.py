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
