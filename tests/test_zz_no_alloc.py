"""The allocation-free entry point (kinc_sim_execute_block_noalloc).

It serves callers that may not allocate device memory -- hosts whose own pool
allocator owns the device and forbids raw cudaMalloc, or code running where
allocating is not allowed.  This test calls it through the C ABI twice in a
row and requires the same K, labels and correlations (bit for bit, the
tolerance of every parity test here) as the allocating entry point.  It lives
in a file of its own, collected last, and works alone in a fresh process as
well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

from kinc_gb300 import Similarity, _native, synthetic

pytestmark = pytest.mark.gpu

CASES = [
    ("gmm_spearman_prepost", 2, 60, 120, dict(clusmethod="gmm", corrmethod="spearman", crit="BIC", preout=True,
                                              postout=True)),
    ("none_pearson", 1, 300, 50, dict()),
    ("kmeans_pearson", 4, 40, 400, dict(clusmethod="kmeans", corrmethod="pearson", maxclus=3, crit="BIC")),
    ("gmm_both_icl", 5, 50, 200, dict(clusmethod="gmm", corrmethod="both", crit="ICL", preout=True,
                                      postout=True)),
    ("none_spearman_3000_samples", 1, 24, 3000, dict(corrmethod="spearman")),
]


def _run_noalloc(L, d_gem, G, S, params, start, size, maxk):
    import torch
    dK = torch.empty(size, dtype=torch.int8, device="cuda")
    dL = torch.empty((size, S), dtype=torch.int8, device="cuda")
    dC = torch.empty((size, maxk, 2) if params.corr_method == 2 else (size, maxk), dtype=torch.float32,
                     device="cuda")
    torch.cuda.synchronize()
    vp = ctypes.c_void_p
    rc = L.kinc_sim_execute_block_noalloc(vp(d_gem.data_ptr()), G, S, ctypes.byref(params), start, size,
                                          vp(dK.data_ptr()), vp(dL.data_ptr()), vp(dC.data_ptr()), None)
    _native.check(rc, None)
    return dK.cpu().numpy(), dL.cpu().numpy(), dC.cpu().numpy()


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_allocating_entry_point(case):
    import torch
    name, wl, G, S, args = case
    gem = synthetic.generate(wl, genes=G, samples=S)
    sim = Similarity(gem, **args)
    sim.initialize()
    total = sim.total_pairs()
    ranges = [(0, min(total, 40000)), (min(total, 40000) // 3, min(total, 40000) // 2)]
    want = [sim.execute(None, start=s, size=n) for s, n in ranges]
    params = sim.params
    sim.close()
    L = _native.load()
    d_gem = torch.from_numpy(gem).cuda()
    for (s, n), w in zip(ranges, want):        # two calls in a row
        K, lab, corr = _run_noalloc(L, d_gem, G, S, params, s, n, params.max_clusters)
        assert np.array_equal(K, w.K)
        multi = w.K > 1
        assert np.array_equal(lab[multi], w.labels[multi])
        assert np.array_equal(np.nan_to_num(corr, nan=9.0), np.nan_to_num(w.corr, nan=9.0))


def test_noalloc_rejects_sizes_beyond_its_limit():
    import torch
    gem = synthetic.generate(1, genes=800, samples=40)
    params = Similarity(gem).params
    L = _native.load()
    d_gem = torch.from_numpy(gem).cuda()
    rc = L.kinc_sim_execute_block_noalloc(ctypes.c_void_p(d_gem.data_ptr()), 800, 40, ctypes.byref(params), 0,
                                          (1 << 18) + 1, None, None, None, None)
    assert rc == _native.EINVAL
    assert b"allocation-free limit" in L.kinc_sim_last_error(None)


def test_noalloc_rejects_work_that_does_not_fit_its_array():
    """GMM k <= 5 at 4,096 samples needs about 4.7 MB of working space per warp: one block of the GMM
    kernel's 20 warps no longer fits the 64 MiB array, so the call is refused before anything runs."""
    import torch
    gem = synthetic.generate(2, genes=40, samples=4096)
    params = Similarity(gem, clusmethod="gmm", corrmethod="spearman", maxclus=5).params
    L = _native.load()
    d_gem = torch.from_numpy(gem).cuda()
    d_out = torch.empty(1 << 16, dtype=torch.uint8, device="cuda")
    vp = ctypes.c_void_p
    rc = L.kinc_sim_execute_block_noalloc(vp(d_gem.data_ptr()), 40, 4096, ctypes.byref(params), 0, 10,
                                          vp(d_out.data_ptr()), vp(d_out.data_ptr()), vp(d_out.data_ptr()), None)
    assert rc == _native.EINVAL
    assert b"do not fit" in L.kinc_sim_last_error(None)
