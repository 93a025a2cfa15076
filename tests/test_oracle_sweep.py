"""Randomised parity sweeps of the C restatement (oracle/kinc_oracle.c) against
KINC's own code compiled by oracle/build_ref.py (skipped without the KINC tree).

Each case draws a workload (kinc_gb300.synthetic 1, 2, 4 or 5), a matrix shape and
every argument of the analytic (clustering none / GMM / K-means, Pearson /
Spearman, BIC / ICL, pre and post outliers, cluster range, minsamp, minexpr), runs
the first pairs of the matrix through both and compares K, N, the labels of
multi-cluster pairs and every correlation bit for bit.  The OpenCL sweep runs the
restatement in rand="lcg" mode against KINC's OpenCL kernels (clustering none or
GMM; minexpr integral, as that worker passes it as an int; Pearson correlations
only of pairs with no excluded sample, the others reading the worker's stale slot
contents).  KINC_SWEEP_CASES sets the number of cases (default 12 each).
"""
import os

import numpy as np
import pytest

from kinc_gb300 import synthetic
from oracle import pyoracle

pytestmark = pytest.mark.slow
CASES = int(os.environ.get("KINC_SWEEP_CASES", "12"))
PAIRS = 200


def same_corr(a, b):
    return np.array_equal(np.nan_to_num(a, nan=9.0), np.nan_to_num(b, nan=9.0))


def random_case(rng):
    wl = int(rng.choice([1, 2, 4, 5]))
    G = int(rng.integers(20, 60))
    S = int(rng.integers(25, 420))
    clus = int(rng.integers(0, 3))
    kw = dict(clus_method=clus, corr_method=int(rng.integers(0, 2)), criterion=int(rng.integers(0, 2)),
              pre_out=int(rng.integers(0, 2)), post_out=int(rng.integers(0, 2)),
              min_clusters=int(rng.integers(1, 3)),
              max_clusters=int(rng.integers(2, 6)) if clus != 2 else int(rng.integers(2, 4)),
              min_samples=int(rng.integers(15, 40)), min_expr=float(rng.choice([-np.inf, 5.0, 6.5])))
    if kw["min_clusters"] > kw["max_clusters"]:
        kw["min_clusters"] = 1
    gem = synthetic.generate(wl, genes=G, samples=S, seed=int(rng.integers(1 << 30)))
    return wl, gem, kw


@pytest.mark.parametrize("case", range(CASES))
def test_sweep_serial(case):
    if pyoracle.ref_lib(0) is None:
        pytest.skip("KINC source tree not present")
    rng = np.random.default_rng(123 + case)
    wl, gem, kw = random_case(rng)
    G, S = gem.shape
    size = min(G * (G - 1) // 2, PAIRS)
    p = pyoracle.params(**kw)
    a = pyoracle.run_block(gem, p, 0, size)
    b = pyoracle.run_ref(gem, p, 0, size)
    info = f"workload {wl}, {G} x {S}, {kw}"
    assert np.array_equal(a[0], b[0]), info
    assert np.array_equal(a[3], b[3]), info
    assert np.array_equal(a[1][a[0] > 1], b[1][b[0] > 1]), info
    assert same_corr(a[2], b[2]), info


@pytest.mark.parametrize("case", range(CASES))
def test_sweep_opencl(case):
    if pyoracle.ocl_lib() is None:
        pytest.skip("KINC source tree not present")
    rng = np.random.default_rng(5000 + case)
    wl, gem, kw = random_case(rng)
    kw["clus_method"] = int(rng.integers(0, 2))                   # none or GMM
    kw["max_clusters"] = max(kw["max_clusters"], kw["min_clusters"])
    kw["min_expr"] = float(rng.choice([-np.inf, 5.0, 6.0]))       # integral, as the worker passes it
    G, S = gem.shape
    size = min(G * (G - 1) // 2, PAIRS)
    p = pyoracle.params(rand_mode=1, **kw)
    K1, L1, C1, N1 = pyoracle.run_block(gem, p, 0, size)
    K2, L2, C2 = pyoracle.run_ocl(gem, p, 0, size, ksize=int(rng.choice([32, 256, 4096])))
    rows = np.ones(size, bool) if p.corr_method == 1 else (N1 == S)
    mask = rows[:, None] & (np.arange(p.max_clusters)[None, :] < K1[:, None])
    info = f"workload {wl}, {G} x {S}, {kw}"
    assert np.array_equal(K1, K2), info
    assert np.array_equal(L1[K1 > 1], L2[K1 > 1]), info
    assert same_corr(C1[mask], C2[mask]), info
