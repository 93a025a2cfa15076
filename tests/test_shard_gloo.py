"""Multi-process sharding of the Similarity path on CPU: world_size 2 over
gloo.  Each rank runs its contiguous range of work blocks (on the oracle --
the per-pair computation is the same on every worker), the item lists are
gathered to rank 0 and merged in rank order, and the result equals a
single-process run.  No GPU is involved."""
import os
import socket

import numpy as np
import pytest

from kinc_gb300 import shard, synthetic


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _items(gem, start, size, kw):
    from oracle import pyoracle
    p = pyoracle.params(**kw)
    if size == 0:
        return {"x": [], "y": [], "c": [], "r": []}, {"x": [], "y": [], "c": [], "codes": []}
    K, labels, corr, _ = pyoracle.run_block(gem, p, start, size)
    cmx, ccm = pyoracle.process_block(gem.shape[1], p, start, K, labels, corr)
    return ({k: v.tolist() for k, v in cmx.items()},
            {"x": ccm["x"].tolist(), "y": ccm["y"].tolist(), "c": ccm["c"].tolist(),
             "codes": [row.tobytes() for row in ccm["codes"]]})


def _worker(rank, world, port, genes, samples, kw, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    gem = synthetic.generate(2, genes=genes, samples=samples)
    kw = dict(kw)
    if kw.pop("by_cost", False):
        sh = shard.shard_pairs_by_cost(shard.block_costs(gem, block=128), genes, world, rank, block=128)
    else:
        sh = shard.shard_pairs(genes, world, rank, block=128)
    mine = _items(gem, sh.start, sh.size, kw)
    gathered = [None] * world
    dist.all_gather_object(gathered, (sh.start, sh.size, mine))
    if rank == 0:
        q.put(gathered)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("kw", [dict(clus_method=1, corr_method=0, criterion=0, post_out=1),
                                dict(clus_method=0, corr_method=1),
                                dict(clus_method=1, corr_method=1, criterion=1, by_cost=True)])
def test_two_ranks_equal_one(kw):
    import torch.multiprocessing as mp
    genes, samples, world = 28, 60, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, genes, samples, kw, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    # shards are contiguous, disjoint and cover every pair
    ranges = [(g[0], g[1]) for g in gathered]
    assert ranges[0][0] == 0 and ranges[0][0] + ranges[0][1] == ranges[1][0]
    assert ranges[1][0] + ranges[1][1] == shard.total_pairs(genes)
    cmx = shard.merge_items([g[2][0] for g in gathered])
    ccm = shard.merge_items([g[2][1] for g in gathered])
    gem = synthetic.generate(2, genes=genes, samples=samples)
    one_cmx, one_ccm = _items(gem, 0, shard.total_pairs(genes), {k: v for k, v in kw.items() if k != "by_cost"})
    for k in one_cmx:
        assert list(cmx[k]) == list(one_cmx[k]), k
    for k in one_ccm:
        assert list(ccm[k]) == list(one_ccm[k]), k


def _write_files(path_ccm, path_cmx, genes, samples, maxk, cmx, ccm):
    from kinc_gb300 import pairwise_matrix as pm
    pm.write(path_cmx, pm.CMX, genes, maxk, 1, cmx["x"], cmx["y"], cmx["c"],
             np.array(cmx["r"], np.float32).reshape(-1, 1))
    codes = np.frombuffer(b"".join(ccm["codes"]), np.int8).reshape(-1, samples)
    pm.write(path_ccm, pm.CCM, genes, maxk, samples, ccm["x"], ccm["y"], ccm["c"], codes)


def _file_worker(rank, world, port, genes, samples, kw, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    gem = synthetic.generate(2, genes=genes, samples=samples)
    sh = shard.shard_pairs_by_cost(shard.block_costs(gem, block=64), genes, world, rank, block=64)
    cmx, ccm = _items(gem, sh.start, sh.size, kw)
    _write_files(os.path.join(out_dir, f"r{rank}.ccm"), os.path.join(out_dir, f"r{rank}.cmx"), genes, samples,
                 kw.get("max_clusters", 5), cmx, ccm)
    dist.barrier()
    dist.destroy_process_group()


def test_rank_files_merge_into_the_single_run_files(tmp_path, native):
    """Each of three ranks writes the CCM/CMX files of its range of work blocks; joined in rank
    order (kinc_pm_concat) they are byte for byte the files of a single-process run."""
    import torch.multiprocessing as mp

    from kinc_gb300 import pairwise_matrix as pm
    genes, samples, world = 30, 50, 3
    kw = dict(clus_method=1, corr_method=1, criterion=0, pre_out=1)
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_file_worker, args=(r, world, port, genes, samples, kw, str(tmp_path)))
             for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    for ext in ("ccm", "cmx"):
        pm.concat(tmp_path / f"all.{ext}", [tmp_path / f"r{r}.{ext}" for r in range(world)])
    gem = synthetic.generate(2, genes=genes, samples=samples)
    cmx, ccm = _items(gem, 0, shard.total_pairs(genes), kw)
    _write_files(tmp_path / "one.ccm", tmp_path / "one.cmx", genes, samples, 5, cmx, ccm)
    for ext in ("ccm", "cmx"):
        assert (tmp_path / f"all.{ext}").read_bytes() == (tmp_path / f"one.{ext}").read_bytes(), ext


def test_shards_cover_all_pairs():
    for genes in (2, 3, 100, 5000):
        for world in (1, 2, 3, 8):
            shards = [shard.shard_pairs(genes, world, r) for r in range(world)]
            assert shards[0].start == 0
            assert all(a.end == b.start for a, b in zip(shards, shards[1:]))
            assert shards[-1].end == shard.total_pairs(genes)
            assert all(s.start % shard.WORK_BLOCK_SIZE == 0 for s in shards if s.size)


def test_block_costs_estimate_pairwise_counts():
    """The per-block cost proxy (n_x n_y / S summed over the block's pairs) tracks the true
    pairwise usable counts on a matrix with per-gene missing rates (uneven workload)."""
    gem = synthetic.generate(4, genes=300, samples=200)
    costs = shard.block_costs(gem, block=256)
    u = ~np.isnan(gem)
    x, y = np.tril_indices(gem.shape[0], -1)
    order = np.lexsort((y, x))
    true = (u[x[order]] & u[y[order]]).sum(axis=1)
    per_block = np.add.reduceat(true, np.arange(0, len(true), 256))
    assert np.allclose(costs, per_block, rtol=0.05)
    assert abs(costs.sum() / true.sum() - 1) < 1e-3


@pytest.mark.parametrize("world", [2, 3, 5])
def test_cost_shards_cover_and_balance(world):
    gem = synthetic.generate(4, genes=500, samples=150)
    G = gem.shape[0]
    costs = shard.block_costs(gem, block=512)
    shs = [shard.shard_pairs_by_cost(costs, G, world, r, block=512) for r in range(world)]
    assert shs[0].start == 0 and shs[-1].end == G * (G - 1) // 2
    assert all(a.end == b.start for a, b in zip(shs, shs[1:]))
    assert all(s.start % 512 == 0 for s in shs)
    share = [costs[s.start // 512:(s.end + 511) // 512].sum() / costs.sum() for s in shs]
    by_count = [shard.shard_pairs(G, world, r, block=512) for r in range(world)]
    share_count = [costs[s.start // 512:(s.end + 511) // 512].sum() / costs.sum() for s in by_count]
    assert max(share) - min(share) <= max(share_count) - min(share_count) + 1e-12
    assert max(share) - 1 / world < 2 * costs.max() / costs.sum()


@pytest.mark.parametrize("by_cost", [False, True])
def test_native_shards_equal_the_python_cuts(native, by_cost):
    """kinc_shard_blocks cuts where shard_pairs / shard_pairs_by_cost cut at KINC's block size."""
    gem = synthetic.generate(4, genes=900, samples=60)
    G = gem.shape[0]
    costs = shard.block_costs(gem, min_expr=5.0) if by_cost else None
    for world in (1, 2, 3, 5, 8):
        got = []
        for rank in range(world):
            first, n = shard.shard_blocks(gem, world, rank, by_cost=by_cost, min_expr=5.0)
            want = (shard.shard_pairs_by_cost(costs, G, world, rank) if by_cost
                    else shard.shard_pairs(G, world, rank))
            assert first * shard.WORK_BLOCK_SIZE == want.start
            assert min((first + n) * shard.WORK_BLOCK_SIZE, shard.total_pairs(G)) == want.end
            got.append((first, n))
        assert got[0][0] == 0 and all(a[0] + a[1] == b[0] for a, b in zip(got, got[1:]))
        assert sum(n for _, n in got) == -(-shard.total_pairs(G) // shard.WORK_BLOCK_SIZE)
    with pytest.raises(ValueError):
        shard.shard_blocks(gem, 2, 2)
