"""Parity at the workloads' full sizes: the worker holds the whole matrix (5,000 x 1,000,
10,000 x 4,000, 30,000 x 500, 20,000 x 2,000) and samples of its pairs -- whole-work-block
starts drawn at random, the matrix's last (ragged) work block, the middle of the largest
workload -- are compared with the oracle bit for bit, and the tensor-core correlations with
the FP64 oracle at the precision target (max |r - r_FP64| <= 1e-4)."""
import ctypes

import numpy as np
import pytest

from kinc_gb300 import Similarity, _native, synthetic
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _segments(total, n, size, seed, last=True):
    rng = np.random.default_rng(seed)
    nblocks = (total + 32767) // 32768
    starts = [int(b) * 32768 for b in rng.choice(nblocks - 1, size=n, replace=False)]
    if last:
        starts.append((nblocks - 1) * 32768)
    return [(s, min(size, total - s)) for s in starts]


def _check(sim, gem, oargs, segments, col=None):
    for start, size in segments:
        res = sim.execute(None, start=start, size=size)
        K, labels, corr, _ = pyoracle.run_block(gem, pyoracle.params(**oargs), start, size)
        assert np.array_equal(res.K, K), f"K differs at {start}"
        multi = K > 1
        assert np.array_equal(res.labels[multi], labels[multi]), f"labels differ at {start}"
        got = res.corr if col is None else res.corr[:, :, col]
        assert np.array_equal(np.nan_to_num(got, nan=9.0), np.nan_to_num(corr, nan=9.0)), f"r differs at {start}"


def test_gmm_spearman_5000x1000():
    gem = synthetic.generate(2)
    sim = Similarity(gem, clusmethod="gmm", corrmethod="spearman", crit="BIC", preout=True, postout=True)
    sim.initialize()
    _check(sim, gem, dict(clus_method=1, corr_method=1, criterion=0, pre_out=1, post_out=1),
           _segments(sim.total_pairs(), 3, 40, seed=101))
    sim.close()


def test_kmeans_pearson_10000x4000():
    gem = synthetic.generate(4)
    sim = Similarity(gem, clusmethod="kmeans", corrmethod="pearson", crit="BIC", maxclus=3)
    sim.initialize()
    _check(sim, gem, dict(clus_method=2, corr_method=0, criterion=0, max_clusters=3),
           _segments(sim.total_pairs(), 2, 6, seed=102))
    sim.close()


def test_gmm_icl_both_30000x500_middle():
    """corrmethod both on the largest matrix: column 0 equals the oracle's Pearson run, column 1 its
    Spearman run, on a segment from the middle of the 449,985,000 pairs."""
    gem = synthetic.generate(5)
    sim = Similarity(gem, clusmethod="gmm", corrmethod="both", crit="ICL", preout=True, postout=True)
    sim.initialize()
    mid = (sim.total_pairs() // 2) // 32768 * 32768
    segs = [(mid, 24)]
    base = dict(clus_method=1, criterion=1, pre_out=1, post_out=1)
    _check(sim, gem, dict(base, corr_method=0), segs, col=0)
    _check(sim, gem, dict(base, corr_method=1), segs, col=1)
    sim.close()


@pytest.mark.parametrize("precision,tol", [("tf32", 1e-4), ("3xbf16", 1e-5), ("fp16", 1e-4)])
def test_tensor_core_20000x2000_vs_fp64(precision, tol):
    gem = synthetic.generate(3)
    sim = Similarity(gem, semantics="fixed", precision=precision)
    sim.initialize()
    L = _native.load()
    total = sim.total_pairs()
    worst = 0.0
    for start, size in _segments(total, 2, 200_000, seed=103):
        K = np.empty(size, np.int8)
        corr = np.empty((size, sim.params.max_clusters), np.float32)
        rc = L.kinc_sim_execute_block(sim._ctx, start, size, K.ctypes.data_as(ctypes.c_void_p), None,
                                      corr.ctypes.data_as(ctypes.c_void_p))
        _native.check(rc, sim._ctx)
        x, y = pyoracle.pair_xy(np.arange(start, start + size))
        ref = pyoracle.pearson_fp64_pairs(gem, x, y)
        got = corr[:, 0].astype(np.float64)
        assert np.array_equal(np.isnan(got), np.isnan(ref))
        ok = ~np.isnan(ref)
        worst = max(worst, float(np.abs(got[ok] - ref[ok]).max()))
    sim.close()
    assert worst <= tol, f"max |r - r_fp64| = {worst}"
