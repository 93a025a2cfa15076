"""GPU parity: the CUDA worker against the oracle (the C restatement of the
reference's serial path, itself pinned to KINC's compiled Pairwise:: code by
test_oracle.py).  Integer outputs (K, N, labels) and correlations must match
bit for bit: the worker repeats the reference's float operation sequence."""
import numpy as np
import pytest

from kinc_gb300 import Similarity, synthetic
from oracle import pyoracle

pytestmark = pytest.mark.gpu

CASES = [
    # name, workload, genes, samples, start, size, gpu args, oracle args
    ("gmm_spearman_bic_outliers", 2, 60, 120, 0, 1770,
     dict(clusmethod="gmm", corrmethod="spearman", crit="BIC", preout=True, postout=True),
     dict(clus_method=1, corr_method=1, criterion=0, pre_out=1, post_out=1)),
    ("gmm_pearson_icl", 2, 60, 120, 100, 900,
     dict(clusmethod="gmm", corrmethod="pearson", crit="ICL"),
     dict(clus_method=1, corr_method=0, criterion=1)),
    ("kmeans_pearson_bic", 4, 50, 160, 0, 1225,
     dict(clusmethod="kmeans", corrmethod="pearson", crit="BIC", maxclus=3),
     dict(clus_method=2, corr_method=0, criterion=0, max_clusters=3)),
    ("none_pearson", 1, 300, 50, 0, 44850, dict(), dict()),
    # ten work blocks from inside the second one: links searched by several CTAs per work block,
    # packed-array reads of the one-thread-per-pair kernel, S above one mask word with a ragged tail
    ("none_pearson_many_blocks", 1, 800, 100, 50000, 200000, dict(), dict()),
    ("none_pearson_fixed_many_blocks", 1, 800, 100, 50000, 200000, dict(semantics="fixed"), dict(semantics=1)),
    ("none_pearson_minexpr", 1, 400, 45, 1000, 60000, dict(minexpr=7.0), dict(min_expr=7.0)),
    ("none_spearman", 1, 200, 70, 0, 19900, dict(corrmethod="spearman"), dict(corr_method=1)),
    ("gmm_pearson_fixed_lcg", 2, 50, 100, 0, 1225,
     dict(clusmethod="gmm", corrmethod="pearson", crit="BIC", semantics="fixed", rand="lcg", postout=True),
     dict(clus_method=1, corr_method=0, criterion=0, semantics=1, rand_mode=1, post_out=1)),
]


def _corr_equal(a, b):
    return np.array_equal(np.nan_to_num(a, nan=9.0), np.nan_to_num(b, nan=9.0))


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_gpu_matches_oracle(case):
    name, wl, G, S, start, size, gargs, oargs = case
    gem = synthetic.generate(wl, genes=G, samples=S)
    sim = Similarity(gem, **gargs)
    sim.initialize()
    size = min(size, sim.total_pairs() - start)
    res = sim.execute(None, start=start, size=size)
    sim.close()
    K, labels, corr, N = pyoracle.run_block(gem, pyoracle.params(**oargs), start, size)
    assert np.array_equal(res.K, K), f"K differs on {(res.K != K).sum()} pairs"
    multi = K > 1
    assert np.array_equal(res.labels[multi], labels[multi])
    diff = np.abs(np.nan_to_num(res.corr, nan=9.0) - np.nan_to_num(corr, nan=9.0))
    assert _corr_equal(res.corr, corr), f"max |dr| {diff.max()} on {(diff > 0).sum()} entries"


@pytest.mark.parametrize("clus", ["gmm", "kmeans", "none"])
def test_both_correlations_equal_single_method_runs(clus):
    """corrmethod both: column 0 equals the Pearson run, column 1 the Spearman run, bit for bit."""
    gem = synthetic.generate(5, genes=50, samples=90)
    args = dict(clusmethod=clus, crit="ICL", preout=True, postout=True, maxclus=4)
    runs = {}
    for method in ("pearson", "spearman", "both"):
        sim = Similarity(gem, corrmethod=method, **args)
        sim.initialize()
        runs[method] = sim.execute(None, start=0, size=sim.total_pairs())
        sim.close()
    both = runs["both"]
    assert both.corr.shape[-1] == 2
    assert np.array_equal(both.K, runs["pearson"].K)
    assert _corr_equal(both.corr[..., 0], runs["pearson"].corr)
    assert _corr_equal(both.corr[..., 1], runs["spearman"].corr)


def test_execute_block_async_equals_execute_block():
    """kinc_sim_execute_block_async into pinned host arrays, completed by kinc_sim_synchronize, returns
    what the synchronous entry point returns."""
    import ctypes

    import torch

    from kinc_gb300 import _native
    gem = synthetic.generate(2, genes=70, samples=90)
    sim = Similarity(gem, clusmethod="gmm", corrmethod="spearman", crit="BIC", postout=True)
    sim.initialize()
    L = _native.load()
    start, size = 100, 1500
    want = sim.execute(None, start=start, size=size)
    K = torch.empty(size, dtype=torch.int8, pin_memory=True)
    lab = torch.empty((size, 90), dtype=torch.int8, pin_memory=True)
    corr = torch.empty((size, 5), dtype=torch.float32, pin_memory=True)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    _native.check(L.kinc_sim_execute_block_async(sim._ctx, start, size, vp(K), vp(lab), vp(corr)), sim._ctx)
    _native.check(L.kinc_sim_synchronize(sim._ctx), sim._ctx)
    sim.close()
    assert np.array_equal(K.numpy(), want.K)
    multi = want.K > 1
    assert np.array_equal(lab.numpy()[multi], want.labels[multi])
    assert _corr_equal(corr.numpy(), want.corr)
