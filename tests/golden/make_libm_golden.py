"""Generate tests/golden/libm/*.npz: KINC's own CPU code built against the C
library's exp/log, on seeded matrices of the clustering workloads.

KINC's GMM calls unqualified exp() and log() on float arguments
(src/core/pairwise_gmm.cpp:177,219,262,271,356).  Which functions those are
depends on the headers of the build: glibc's float expf/logf (math mode 1) or
its double exp/log with the surrounding sums partly in double (math mode 2).
The bit-exact fixtures next to this script pin mode 0 (kinc_expf/kinc_logf,
the functions the GPU and the oracle use); these fixtures record what the two
library builds give on the same inputs, so tests and the benchmark can report
how closely the GPU agrees with KINC as it is usually built.

Each case is a 64-gene matrix (2,016 pairs, all in one work block, computed
in one serial pass) with the workload's full sample count and value
distributions (kinc_gb300.synthetic with genes=64), run with the workload's
arguments:

* gmm_spearman_5000x1000:  GMM k 1..5, BIC, pre+post outliers, Spearman;
* kmeans_pearson_10000x4000: K-means k 1..3, BIC, Pearson;
* gmm_both_icl_30000x500:  GMM k 1..5, ICL, pre+post outliers, Pearson and
  Spearman (two runs of KINC's code, one per correlation, as KINC computes one
  method per run).

Stored per mode m in (0, 1, 2): K, correlations and a blake2b-64 hash of
every pair's label row; for modes 1 and 2 also the full label rows of the
pairs whose labels differ from mode 0 (so sample-level agreement can be
counted).  Mode 0 is a bit-exact target like the other fixtures here.  Regenerate with the
KINC tree present:

    KINC_REFERENCE_DIR=/path/to/KINC python tests/golden/make_libm_golden.py
"""
import hashlib
import json
import os
import sys
from multiprocessing import get_context

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

OUT = os.path.join(HERE, "libm")
GENES = 64

# name: (workload, [oracle params per run]; two runs are stacked as the two correlations of corrmethod both)
CASES = {
    "gmm_spearman_5000x1000": (2, [dict(clus_method=1, corr_method=1, criterion=0, pre_out=1, post_out=1,
                                        max_clusters=5)]),
    "kmeans_pearson_10000x4000": (4, [dict(clus_method=2, corr_method=0, criterion=0, max_clusters=3)]),
    "gmm_both_icl_30000x500": (5, [dict(clus_method=1, corr_method=0, criterion=1, pre_out=1, post_out=1,
                                        max_clusters=5),
                                   dict(clus_method=1, corr_method=1, criterion=1, pre_out=1, post_out=1,
                                        max_clusters=5)]),
}


def row_hashes(labels):
    """blake2b-64 of each int8 label row, as uint64."""
    return np.array([int.from_bytes(hashlib.blake2b(r.tobytes(), digest_size=8).digest(), "little")
                     for r in np.ascontiguousarray(labels, np.int8)], dtype=np.uint64)


def _job(args):
    wl, kw, mode, start, size = args
    from kinc_gb300 import synthetic
    from oracle import pyoracle
    gem = synthetic.generate(wl, genes=GENES)
    out = pyoracle.run_ref(gem, pyoracle.params(**kw), start, size, math_mode=mode)
    if out is None:
        raise SystemExit("the KINC source tree is required to generate these fixtures")
    return out


def run_all(pool, wl, runs, total):
    """Every mode and run over all pairs, each as one call from pair 0 (one work block, so the
    reference's Pearson reads the same stale packed values as in a serial run)."""
    keys = [(mode, j) for mode in (0, 1, 2) for j in range(len(runs))]
    outs = pool.map(_job, [(wl, runs[j], mode, 0, total) for mode, j in keys])
    return dict(zip(keys, outs))


def make(pool, name):
    from kinc_gb300 import synthetic
    wl, runs = CASES[name]
    gem = synthetic.generate(wl, genes=GENES)
    total = GENES * (GENES - 1) // 2
    everything = run_all(pool, wl, runs, total)
    res = {}
    for mode in (0, 1, 2):
        outs = [everything[(mode, j)] for j in range(len(runs))]
        K, labels, _, N = outs[0]
        for o in outs[1:]:
            assert np.array_equal(o[0], K) and np.array_equal(o[1], labels)
        corr = outs[0][2] if len(outs) == 1 else np.stack([o[2] for o in outs], axis=-1)
        res[mode] = (K, labels, corr, N)
    store = dict(gem=gem, N=res[0][3], params=json.dumps(runs[0]), ncorr=np.int32(len(runs)))
    h0 = row_hashes(res[0][1])
    store.update(K0=res[0][0], corr0=res[0][2], hash0=h0)
    for mode in (1, 2):
        K, labels, corr, N = res[mode]
        assert np.array_equal(N, res[0][3])
        h = row_hashes(labels)
        diff = np.nonzero(h != h0)[0].astype(np.int32)
        store.update({f"K{mode}": K, f"corr{mode}": corr, f"hash{mode}": h, f"diff{mode}": diff,
                      f"labels{mode}": labels[diff]})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **store)
    return res


if __name__ == "__main__":
    os.makedirs(OUT, exist_ok=True)
    only = sys.argv[1:]
    with get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        for n in CASES:
            if not only or n in only:
                res = make(pool, n)
                K0 = res[0][0]
                print(f"{n}: {len(K0)} pairs, K histogram (mode 0) {np.bincount(K0.astype(np.int64)).tolist()}")
