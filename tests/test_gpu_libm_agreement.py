"""GPU results on the clustering workloads' 64-gene matrices (tests/golden/libm/,
2,016 pairs each, every pair in one call): bit-exact against KINC's own code in
math mode 0, and the agreement with KINC built against glibc's float (mode 1)
and double (mode 2) exp/log, which is reported and held to the bounds the
library builds keep with each other (tests/test_libm_agreement.py)."""
import json

import numpy as np
import pytest

from kinc_gb300 import Similarity
from oracle import agreement

pytestmark = pytest.mark.gpu

CASES = agreement.cases()
NAMES = {0: "none", 1: "gmm", 2: "kmeans"}


def run_gpu(fx):
    a = fx["params"]
    sim = Similarity(fx["gem"], clusmethod=NAMES[a["clus_method"]],
                     corrmethod=2 if fx["ncorr"] == 2 else a["corr_method"], minsamp=a.get("min_samples", 30),
                     minclus=a.get("min_clusters", 1), maxclus=a["max_clusters"], crit=a["criterion"],
                     preout=a.get("pre_out", 0), postout=a.get("post_out", 0))
    sim.initialize()
    res = sim.execute(None, start=0, size=len(fx["K0"]))
    sim.close()
    return res


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_bit_exact_mode0_and_agreement(name, record_property):
    fx = agreement.load(CASES[name])
    res = run_gpu(fx)
    # bit-exact against KINC's own code with the portable exp/log, all 2,016 pairs
    assert np.array_equal(res.K, fx["K0"]), f"K differs on {(res.K != fx['K0']).sum()} pairs"
    h = agreement.row_hashes(res.labels)
    assert np.array_equal(h, fx["hash0"]), f"label rows differ on {(h != fx['hash0']).sum()} pairs"
    assert np.array_equal(np.nan_to_num(res.corr, nan=9.0).view(np.uint32),
                          np.nan_to_num(fx["corr0"], nan=9.0).view(np.uint32))
    for mode in (1, 2):
        st = agreement.compare(res.K, res.labels, res.corr, fx, mode)
        record_property(f"mode{mode}", json.dumps(st))
        print(name, json.dumps(st))
        assert st["k_agreement"] >= 0.95, st
        assert st["label_agreement"] >= 0.7, st
        assert st["sample_label_agreement"] >= 0.999, st
        assert st["rows_without_reference"] == 0, st
        assert st["nan_mismatches"] == 0, st
        assert st["max_abs_dr_same_labels"] <= 1e-5, st
