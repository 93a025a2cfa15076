"""The rand="lcg" mode pinned against KINC's OpenCL worker: its kernels (src/opencl/*.cl)
compiled for the host and driven like Similarity::OpenCL::Worker (oracle/build_ref.py,
oracle/ocl_driver.cpp).  The restatement in that mode must give the same K, the same labels
and the same correlations; the GPU is held to the same outputs through the ocl_* golden
fixtures (tests/test_gpu_golden.py).  Needs the KINC tree to build the kernels; skipped
without it."""
import numpy as np
import pytest

from kinc_gb300 import synthetic
from oracle import pyoracle

from test_oracle import same_corr


def _need_ocl():
    if pyoracle.ocl_lib() is None:
        pytest.skip("KINC source tree not present: OpenCL kernels not built")


def _usable(gem, min_expr, start, size):
    G = gem.shape[0]
    ok = ~np.isnan(gem) & ~(gem < np.float32(min_expr))
    xs, ys = np.tril_indices(G, -1)
    return (ok[xs[start:start + size]] & ok[ys[start:start + size]]).sum(axis=1)


def _compare(gem, kw, start=0, size=None, ksize=64):
    G, S = gem.shape
    size = G * (G - 1) // 2 - start if size is None else size
    p = pyoracle.params(rand_mode=1, **kw)
    K1, L1, C1, _ = pyoracle.run_block(gem, p, start, size)
    K2, L2, C2 = pyoracle.run_ocl(gem, p, start, size, ksize=ksize)
    assert np.array_equal(K1, K2), f"K differs on {(K1 != K2).sum()} of {size} pairs"
    multi = K1 > 1
    assert np.array_equal(L1[multi], L2[multi])
    # correlations of the clusters below K, on the pairs whose values the OpenCL Pearson kernel
    # determines (Spearman: every pair; Pearson: pairs with no excluded sample)
    rows = np.ones(size, bool) if p.corr_method == 1 else _usable(gem, p.min_expr, start, size) == S
    mask = rows[:, None] & (np.arange(p.max_clusters)[None, :] < K1[:, None])
    assert same_corr(C1[mask], C2[mask])
    return K1, rows


GMM_CASES = [
    dict(clus_method=1, corr_method=1, criterion=0),
    dict(clus_method=1, corr_method=1, criterion=1, pre_out=1, post_out=1),
    dict(clus_method=1, corr_method=0, criterion=0, pre_out=1, post_out=1),
    dict(clus_method=1, corr_method=0, criterion=1, min_clusters=2, max_clusters=4),
    dict(clus_method=1, corr_method=1, criterion=0, min_expr=6.0, post_out=1),
]


CASES = [(kw, False) for kw in GMM_CASES] + [(GMM_CASES[1], True), (GMM_CASES[2], True)]


@pytest.mark.parametrize("kw,complete", CASES,
                         ids=["-".join(f"{k}{v}" for k, v in kw.items()) + ("-complete" if c else "") for kw, c in CASES])
def test_lcg_mode_equals_opencl_kernels(kw, complete):
    _need_ocl()
    gem = synthetic.generate(2, genes=26, samples=60, seed=7)
    if complete:
        gem = np.where(np.isnan(gem), np.float32(8.0), gem).astype(np.float32)
    K, rows = _compare(gem, kw)
    assert (K > 1).any()
    if complete or kw["corr_method"] == 1:
        assert rows.all()


def test_no_clustering_and_work_block_chunks():
    """Chunks of ksize work items inside 32,768-pair work blocks, across a block boundary."""
    _need_ocl()
    gem = synthetic.generate(1, genes=260, samples=40, seed=3)
    _compare(gem, dict(corr_method=1, min_expr=6.0), start=32768 - 300, size=600, ksize=128)
    _compare(gem, dict(corr_method=0), start=32768 - 300, size=600, ksize=4096)
