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


def test_device_process_matches_host_process():
    """kinc_sim_compact_block_device keeps exactly the items kinc_sim_process_pairs keeps."""
    import ctypes

    import torch

    from kinc_gb300 import _native
    gem = synthetic.generate(2, genes=60, samples=75)
    sim = Similarity(gem, clusmethod="gmm", crit="ICL", postout=True, mincorr=0.4)
    sim.initialize()
    L = _native.load()
    total = sim.total_pairs()
    host = sim.execute(None, start=0, size=total)
    S, maxk = 75, 5
    dK = torch.from_numpy(host.K).cuda()
    dL = torch.from_numpy(host.labels).cuda()
    dC = torch.from_numpy(host.corr).cuda()
    cap = total * maxk
    out = [torch.empty(cap, dtype=t, device="cuda") for t in (torch.int32, torch.int32, torch.int8, torch.float32,
                                                              torch.int32, torch.int32, torch.int8)]
    packed = torch.empty((cap, (S + 1) // 2), dtype=torch.uint8, device="cuda")
    counts = torch.zeros(2, dtype=torch.int64, device="cuda")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    torch.cuda.synchronize()
    rc = L.kinc_sim_compact_block_device(sim._ctx, 0, total, vp(dK), vp(dL), vp(dC), vp(out[0]), vp(out[1]),
                                         vp(out[2]), vp(out[3]), cap, vp(out[4]), vp(out[5]), vp(out[6]),
                                         vp(packed), cap, vp(counts), None)
    _native.check(rc, sim._ctx)
    _native.check(L.kinc_sim_synchronize(sim._ctx), sim._ctx)
    n_cmx, n_ccm = counts.cpu().tolist()
    sim.process(host)
    x, y, c, r = sim.cmx.arrays()
    assert n_cmx == len(x)
    assert np.array_equal(out[0][:n_cmx].cpu().numpy(), x) and np.array_equal(out[2][:n_cmx].cpu().numpy(), c)
    assert np.array_equal(out[3][:n_cmx].cpu().numpy(), r)
    mx, my, mc, codes = sim.ccm.arrays()
    assert n_ccm == len(mx)
    unpacked = np.zeros((n_ccm, S), np.int8)
    pk = packed[:n_ccm].cpu().numpy()
    unpacked[:, 0::2] = pk & 0x0F
    unpacked[:, 1::2] = (pk >> 4)[:, :S // 2]
    assert np.array_equal(unpacked, codes)
    sim.close()
