"""The ordered block runner on the GPU writes the same CCM/CMX items the
reference's process() emits (compared with the oracle's process over the same
blocks)."""
import numpy as np
import pytest

from kinc_gb300 import Similarity, pairwise_matrix as pm, synthetic
from oracle import pyoracle

pytestmark = pytest.mark.gpu

CASES = [
    ("gmm_pearson_bic_post", 2, 44, 90, dict(clusmethod="gmm", crit="BIC", postout=True, mincorr=0.3),
     dict(clus_method=1, criterion=0, post_out=1, min_corr=0.3)),
    ("none_pearson_two_blocks", 1, 260, 36, dict(mincorr=0.2), dict(min_corr=0.2)),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_run_to_files_matches_process(tmp_path, case):
    name, wl, G, S, gargs, oargs = case
    gem = synthetic.generate(wl, genes=G, samples=S)
    sim = Similarity(gem, **gargs)
    ccm_path, cmx_path = tmp_path / "out.ccm", tmp_path / "out.cmx"
    sim.run(ccm_path=ccm_path, cmx_path=cmx_path)
    sim.close()
    p = pyoracle.params(**oargs)
    total = G * (G - 1) // 2
    cmx_want, ccm_want = {"x": [], "y": [], "c": [], "r": []}, {"x": [], "y": [], "c": [], "codes": []}
    for start in range(0, total, 32768):
        size = min(32768, total - start)
        K, labels, corr, _ = pyoracle.run_block(gem, p, start, size)
        cmx, ccm = pyoracle.process_block(S, p, start, K, labels, corr)
        for k in cmx_want:
            cmx_want[k].append(cmx[k])
        for k in ccm_want:
            ccm_want[k].append(ccm[k])
    cmx = pm.read(cmx_path, pm.CMX)
    ccm = pm.read(ccm_path, pm.CCM)
    assert np.array_equal(cmx["x"], np.concatenate(cmx_want["x"]))
    assert np.array_equal(cmx["c"], np.concatenate(cmx_want["c"]))
    assert np.array_equal(cmx["payload"][:, 0], np.concatenate(cmx_want["r"]))
    assert np.array_equal(ccm["x"], np.concatenate(ccm_want["x"]))
    codes = np.concatenate(ccm_want["codes"]) if ccm_want["codes"] else np.zeros((0, S), np.int8)
    assert np.array_equal(ccm["payload"], codes.reshape(-1, S))
    assert len(cmx["x"]) > 0
