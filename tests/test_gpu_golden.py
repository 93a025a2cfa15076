"""GPU against the golden fixtures: outputs of KINC's own compiled Pairwise::
code, and of its OpenCL kernels compiled for the host (the ocl_* fixtures, run
in the rand="lcg" mode), on seeded inputs (tests/golden/make_golden.py).
Bit-exact: K, labels of multi-cluster pairs, N-derived results and every
correlation the reference determines."""
import glob
import os

import numpy as np
import pytest

from kinc_gb300 import Similarity

from test_oracle import load_golden, same_corr

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
NAMES = {0: "none", 1: "gmm", 2: "kmeans"}


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_gpu_reproduces_golden(path):
    g = load_golden(path)
    a = g["params"]
    sim = Similarity(g["gem"], clusmethod=NAMES[a["clus_method"]], corrmethod=a["corr_method"],
                     minexpr=a["min_expr"], minsamp=a["min_samples"], minclus=a["min_clusters"],
                     maxclus=a["max_clusters"], crit=a["criterion"], preout=a["pre_out"], postout=a["post_out"],
                     mincorr=a["min_corr"], maxcorr=a["max_corr"],
                     rand="lcg" if a.get("rand_mode") == 1 else "glibc")
    sim.initialize()
    res = sim.execute(None, start=g["start"], size=g["size"])
    sim.close()
    assert np.array_equal(res.K, g["K"]), f"K differs on {(res.K != g['K']).sum()} pairs"
    assert np.array_equal(res.labels[g["multi"]], g["labels"])
    m = g["corr_mask"]
    assert same_corr(res.corr[m], g["corr"][m])
