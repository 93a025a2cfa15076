"""Generate the golden fixtures in this folder from KINC's own code.

Each fixture is the output of KINC's CPU Pairwise:: models -- compiled
unmodified from the KINC source tree by oracle/build_ref.py and driven like
Similarity::Serial -- on a small seeded synthetic expression matrix.  The
reference tree is only needed to (re)generate them:

    KINC_REFERENCE_DIR=/path/to/KINC python tests/golden/make_golden.py

Stored per case (npz): the matrix, the arguments, K, N, the correlations,
and the labels of the pairs with K > 1.
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
    for n in CASES:
        K = make(n)
        print(f"{n}: {len(K)} pairs, K histogram {np.bincount(K.astype(np.int64))}")
