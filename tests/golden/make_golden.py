"""Generate the golden fixtures in this folder from KINC's own code.

Each fixture is the output of KINC's own code on a small seeded synthetic
expression matrix:

* the plain cases: KINC's CPU Pairwise:: models, compiled unmodified from the
  KINC source tree by oracle/build_ref.py and driven like Similarity::Serial;
* the ocl_* cases: KINC's OpenCL kernels (src/opencl/*.cl) compiled for the
  host by oracle/build_ref.py and driven like its OpenCL worker
  (oracle/ocl_driver.cpp): the per-fit LCG initialisation, which the worker's
  rand="lcg" mode reproduces.

The reference tree is only needed to (re)generate them:

    KINC_REFERENCE_DIR=/path/to/KINC python tests/golden/make_golden.py

Stored per case (npz): the matrix, the arguments, K, N, the correlations,
the labels of the pairs with K > 1, and corr_rows: the pairs whose
correlations the reference determines.  That is every pair, except OpenCL
Pearson on a pair with an excluded sample: that kernel then reads the
leftovers of whichever pair last used its work slot (uninitialised device
memory at first), which depends on the worker's chunking, not on the pair.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from kinc_gb300 import synthetic  # noqa: E402
from oracle import pyoracle  # noqa: E402

# name: (workload, genes, samples, start, size or None for all pairs, oracle params)
CASES = {
    "gmm_spearman_bic_prepost": (2, 40, 80, 0, None,
                                 dict(clus_method=1, corr_method=1, criterion=0, pre_out=1, post_out=1)),
    "gmm_pearson_icl": (2, 40, 80, 0, None, dict(clus_method=1, corr_method=0, criterion=1)),
    "gmm_pearson_icl_prepost_k2to4": (5, 36, 90, 0, None,
                                      dict(clus_method=1, corr_method=0, criterion=1, min_clusters=2,
                                           max_clusters=4, pre_out=1, post_out=1)),
    "kmeans_pearson_bic": (4, 30, 120, 0, None, dict(clus_method=2, corr_method=0, criterion=0, max_clusters=3)),
    "kmeans_spearman_icl_post": (4, 24, 150, 0, None,
                                 dict(clus_method=2, corr_method=1, criterion=1, max_clusters=3, post_out=1)),
    "none_pearson_two_blocks": (1, 260, 36, 0, None, dict()),
    "none_spearman": (1, 60, 60, 0, None, dict(corr_method=1)),
    "none_pearson_minexpr": (1, 80, 64, 0, None, dict(min_expr=6.0)),
    "gmm_pearson_minexpr_bic": (1, 30, 100, 0, None, dict(clus_method=1, corr_method=0, criterion=0,
                                                          min_expr=5.0, min_samples=20)),
}


# name: (workload, genes, samples, start, size or None, ksize, complete, oracle params); rand_mode=1 implied
OCL_CASES = {
    "ocl_gmm_spearman_bic_prepost": (2, 40, 80, 0, None, 64, False,
                                     dict(clus_method=1, corr_method=1, criterion=0, pre_out=1, post_out=1)),
    "ocl_gmm_pearson_icl_prepost": (2, 40, 80, 0, None, 64, False,
                                    dict(clus_method=1, corr_method=0, criterion=1, pre_out=1, post_out=1)),
    "ocl_gmm_pearson_bic_complete": (5, 36, 90, 0, None, 4096, True,
                                     dict(clus_method=1, corr_method=0, criterion=0, min_clusters=2,
                                          max_clusters=4, pre_out=1, post_out=1)),
    "ocl_none_spearman_minexpr": (1, 60, 60, 0, None, 4096, False, dict(corr_method=1, min_expr=6.0)),
    "ocl_gmm_spearman_two_blocks": (2, 260, 40, 32768 - 400, 800, 256, False,
                                    dict(clus_method=1, corr_method=1, criterion=0, post_out=1)),
}


def usable_counts(gem, min_expr, start, size):
    """N per pair: samples where both genes are present and neither is below min_expr."""
    G = gem.shape[0]
    ok = ~np.isnan(gem) & ~(gem < np.float32(min_expr))
    xs, ys = np.tril_indices(G, -1)
    order = np.lexsort((ys, xs))                      # pair index order: x, then y
    xs, ys = xs[order][start:start + size], ys[order][start:start + size]
    return (ok[xs] & ok[ys]).sum(axis=1).astype(np.int32)


def make_ocl(name):
    wl, G, S, start, size, ksize, complete, kw = OCL_CASES[name]
    gem = synthetic.generate(wl, genes=G, samples=S)
    if complete:
        gem = np.where(np.isnan(gem), np.float32(8.0), gem).astype(np.float32)
    p = pyoracle.params(rand_mode=1, **kw)
    total = G * (G - 1) // 2
    size = total - start if size is None else size
    out = pyoracle.run_ocl(gem, p, start, size, ksize=ksize)
    if out is None:
        raise SystemExit("the KINC source tree is required to generate golden fixtures")
    K, labels, corr = out
    N = usable_counts(gem, p.min_expr, start, size)
    corr_rows = np.ones(size, bool) if p.corr_method == 1 else (N == S)
    multi = np.nonzero(K > 1)[0]
    args = dict(pyoracle.DEFAULTS)
    args.update(kw)
    args["rand_mode"] = 1
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), gem=gem, K=K, N=N, corr=corr,
                        multi=multi.astype(np.int32), labels=labels[multi], start=np.int64(start),
                        size=np.int64(size), params=json.dumps(args), corr_rows=corr_rows, ksize=np.int32(ksize))
    return K


def make(name):
    wl, G, S, start, size, kw = CASES[name]
    gem = synthetic.generate(wl, genes=G, samples=S)
    p = pyoracle.params(**kw)
    total = G * (G - 1) // 2
    size = total - start if size is None else size
    out = pyoracle.run_ref(gem, p, start, size, math_mode=0)
    if out is None:
        raise SystemExit("the KINC source tree is required to generate golden fixtures")
    K, labels, corr, N = out
    multi = np.nonzero(K > 1)[0]
    args = dict(pyoracle.DEFAULTS)
    args.update(kw)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), gem=gem, K=K, N=N, corr=corr,
                        multi=multi.astype(np.int32), labels=labels[multi], start=np.int64(start),
                        size=np.int64(size), params=json.dumps(args))
    return K


if __name__ == "__main__":
    only = sys.argv[1:]
    for n in CASES:
        if not only or n in only:
            K = make(n)
            print(f"{n}: {len(K)} pairs, K histogram {np.bincount(K.astype(np.int64))}")
    for n in OCL_CASES:
        if not only or n in only:
            K = make_ocl(n)
            print(f"{n}: {len(K)} pairs, K histogram {np.bincount(K.astype(np.int64))}")
