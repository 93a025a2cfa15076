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
    ("kmeans_spearman_icl", 4, 40, 120, dict(clusmethod="kmeans", corrmethod="spearman", crit="ICL", maxclus=3,
                                             mincorr=0.3),
     dict(clus_method=2, corr_method=1, criterion=1, max_clusters=3, min_corr=0.3)),
    ("none_pearson_two_blocks", 1, 260, 36, dict(mincorr=0.2), dict(min_corr=0.2)),
]


def _oracle_items(gem, p, S):
    """The oracle's process() items over every work block, in order."""
    G = gem.shape[0]
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
    return ({k: np.concatenate(v) for k, v in cmx_want.items()},
            {k: (np.concatenate(v) if v else np.zeros((0, S), np.int8)) for k, v in ccm_want.items()})


def _check_files(cmx_path, ccm_path, cmx_want, ccm_want, S):
    cmx = pm.read(cmx_path, pm.CMX)
    assert np.array_equal(cmx["x"], cmx_want["x"])
    assert np.array_equal(cmx["y"], cmx_want["y"])
    assert np.array_equal(cmx["c"], cmx_want["c"])
    assert np.array_equal(cmx["payload"][:, 0], cmx_want["r"])
    if ccm_path is not None:
        ccm = pm.read(ccm_path, pm.CCM)
        assert np.array_equal(ccm["x"], ccm_want["x"])
        assert np.array_equal(ccm["payload"], ccm_want["codes"].reshape(-1, S))
    assert len(cmx["x"]) > 0


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_run_to_files_matches_process(tmp_path, case):
    name, wl, G, S, gargs, oargs = case
    gem = synthetic.generate(wl, genes=G, samples=S)
    sim = Similarity(gem, **gargs)
    ccm_path, cmx_path = tmp_path / "out.ccm", tmp_path / "out.cmx"
    sim.run(ccm_path=ccm_path, cmx_path=cmx_path)
    sim.close()
    cmx_want, ccm_want = _oracle_items(gem, pyoracle.params(**oargs), S)
    _check_files(cmx_path, ccm_path, cmx_want, ccm_want, S)


def test_run_to_files_two_slots_many_device_blocks(tmp_path):
    """Device blocks of one work block each: the two result slots alternate over
    three blocks and the files equal the single-device-block run byte for byte."""
    G, S = 400, 64
    gem = synthetic.generate(2, genes=G, samples=S)
    args = dict(clusmethod="gmm", crit="ICL", preout=True, postout=True, mincorr=0.3)
    one = Similarity(gem, **args)
    one.run(ccm_path=tmp_path / "a.ccm", cmx_path=tmp_path / "a.cmx")
    one.close()
    many = Similarity(gem, **args)
    many.run(ccm_path=tmp_path / "b.ccm", cmx_path=tmp_path / "b.cmx", device_block=32768)
    many.close()
    for ext in ("ccm", "cmx"):
        assert (tmp_path / f"a.{ext}").read_bytes() == (tmp_path / f"b.{ext}").read_bytes()
    p = pyoracle.params(clus_method=1, criterion=1, pre_out=1, post_out=1, min_corr=0.3)
    cmx_want, ccm_want = _oracle_items(gem, p, S)
    _check_files(tmp_path / "b.cmx", tmp_path / "b.ccm", cmx_want, ccm_want, S)
    # the text export of the files equals the export restated over the oracle's items
    pm.export_text(tmp_path / "b.ccm", tmp_path / "b.cmx", tmp_path / "b.txt")
    want = pyoracle.export_text(dict(x=cmx_want["x"], y=cmx_want["y"], payload=cmx_want["r"].reshape(-1, 1)),
                                dict(x=ccm_want["x"], y=ccm_want["y"], payload=ccm_want["codes"].reshape(-1, S)), S)
    assert (tmp_path / "b.txt").read_text() == want
    # the extracted network (clusters with |r| >= 0.5) equals Extract restated over the oracle's items
    pm.write_emx(tmp_path / "b.emx", gem)
    pm.extract(tmp_path / "b.emx", tmp_path / "b.ccm", tmp_path / "b.cmx", tsv_path=tmp_path / "b.tsv",
               graphml_path=tmp_path / "b.graphml", min_corr=0.5)
    want_tsv, want_gml = pyoracle.extract_network(
        gem, dict(x=cmx_want["x"], y=cmx_want["y"], payload=cmx_want["r"].reshape(-1, 1)),
        dict(x=ccm_want["x"], y=ccm_want["y"], payload=ccm_want["codes"].reshape(-1, S)), S, min_corr=0.5)
    assert (tmp_path / "b.tsv").read_text() == want_tsv
    assert (tmp_path / "b.graphml").read_text() == want_gml


def test_run_to_files_partial_range(tmp_path):
    """first_block / nblocks select work blocks; the files hold exactly their items."""
    G, S = 400, 48
    gem = synthetic.generate(1, genes=G, samples=S)
    sim = Similarity(gem, mincorr=0.2)
    sim.run(cmx_path=tmp_path / "p.cmx", first_block=1, nblocks=1, device_block=32768)
    sim.close()
    p = pyoracle.params(min_corr=0.2)
    K, labels, corr, _ = pyoracle.run_block(gem, p, 32768, 32768)
    cmx, _ = pyoracle.process_block(S, p, 32768, K, labels, corr)
    got = pm.read(tmp_path / "p.cmx", pm.CMX)
    assert np.array_equal(got["x"], cmx["x"]) and np.array_equal(got["y"], cmx["y"])
    assert np.array_equal(got["payload"][:, 0], cmx["r"])


def test_run_to_files_grows_item_buffers(tmp_path):
    """A device block keeping more than 2^21 items (every pair of a 2^22-pair block
    with mincorr 0) makes the runner grow its item buffers and compact again."""
    G, S = 3000, 40
    gem = synthetic.generate(1, genes=G, samples=S)
    sim = Similarity(gem, mincorr=0.0, minsamp=30)
    sim.run(cmx_path=tmp_path / "g.cmx")
    sim.close()
    cmx_want, _ = _oracle_items(gem, pyoracle.params(min_corr=0.0, min_samples=30), S)
    assert len(cmx_want["x"]) > (1 << 21)
    _check_files(tmp_path / "g.cmx", None, cmx_want, None, S)


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


def test_command_line_similarity_and_rmt(tmp_path, capsys):
    """python -m kinc_gb300 run similarity writes the files the Python API writes; run rmt reports the
    threshold the API finds."""
    from kinc_gb300 import __main__ as cli
    from kinc_gb300.rmt import RMT
    G, S = 120, 70
    gem = synthetic.generate(2, genes=G, samples=S)
    pm.write_emx(tmp_path / "g.emx", gem)
    assert cli.main(["run", "similarity", "--input", str(tmp_path / "g.emx"), "--ccm", str(tmp_path / "a.ccm"),
                     "--cmx", str(tmp_path / "a.cmx"), "--clusmethod", "gmm", "--corrmethod", "spearman",
                     "--crit", "BIC", "--preout", "--postout", "true", "--mincorr", "0.3"]) == 0
    sim = Similarity(gem, clusmethod="gmm", corrmethod="spearman", crit="BIC", preout=True, postout=True,
                     mincorr=0.3)
    sim.run(ccm_path=tmp_path / "b.ccm", cmx_path=tmp_path / "b.cmx")
    sim.close()
    for ext in ("ccm", "cmx"):
        assert (tmp_path / f"a.{ext}").read_bytes() == (tmp_path / f"b.{ext}").read_bytes()
    # the native host driver, same arguments
    import subprocess

    from kinc_gb300 import build
    r = subprocess.run([build.CLI, "run", "similarity", "--input", str(tmp_path / "g.emx"),
                        "--ccm", str(tmp_path / "c.ccm"), "--cmx", str(tmp_path / "c.cmx"), "--clusmethod", "gmm",
                        "--corrmethod", "spearman", "--crit", "BIC", "--preout", "--postout", "true",
                        "--mincorr", "0.3"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for ext in ("ccm", "cmx"):
        assert (tmp_path / f"c.{ext}").read_bytes() == (tmp_path / f"b.{ext}").read_bytes()
    Gn, x, y, c, r = synthetic.clique_network(80, 5)
    pm.write(tmp_path / "n.cmx", pm.CMX, Gn, 1, 1, x, y, c, r.reshape(-1, 1))
    capsys.readouterr()
    assert cli.main(["run", "rmt", "--input", str(tmp_path / "n.cmx"), "--log", str(tmp_path / "rmt.log"),
                     "--tstep", "0.01"]) in (0, 1)
    out = capsys.readouterr()
    try:
        t, _ = RMT(tstep=0.01).run(input=tmp_path / "n.cmx")
        assert out.out.strip() == f"threshold: {t:g}"
    except Exception:
        assert "rmt:" in out.err


@pytest.mark.parametrize("by_cost", [False, True])
def test_sharded_command_line_runs_merge_into_the_single_run(tmp_path, by_cost):
    """kinc-gb300 run similarity --world 3 --rank r on each rank, then run merge: the joined
    CCM/CMX files are byte for byte the files of one unsharded run."""
    import subprocess

    from kinc_gb300 import build
    G, S = 400, 48                        # 79,800 pairs: three work blocks
    gem = synthetic.generate(4, genes=G, samples=S)
    pm.write_emx(tmp_path / "g.emx", gem)
    common = ["--input", str(tmp_path / "g.emx"), "--clusmethod", "gmm", "--corrmethod", "pearson", "--crit",
              "BIC", "--postout", "--mincorr", "0.3"]
    r = subprocess.run([build.CLI, "run", "similarity", *common, "--ccm", str(tmp_path / "one.ccm"), "--cmx",
                        str(tmp_path / "one.cmx")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for rank in range(3):
        r = subprocess.run([build.CLI, "run", "similarity", *common, "--ccm", str(tmp_path / f"r{rank}.ccm"),
                            "--cmx", str(tmp_path / f"r{rank}.cmx"), "--world", "3", "--rank", str(rank),
                            *(["--by-cost"] if by_cost else [])], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
    for ext in ("ccm", "cmx"):
        r = subprocess.run([build.CLI, "run", "merge", "--output", str(tmp_path / f"all.{ext}"), "--inputs",
                            ",".join(str(tmp_path / f"r{k}.{ext}") for k in range(3))], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert (tmp_path / f"all.{ext}").read_bytes() == (tmp_path / f"one.{ext}").read_bytes(), ext


@pytest.mark.parametrize("precision", ["tf32", "3xbf16", "fp16"])
def test_run_to_files_tensor_core_matches_execute(tmp_path, precision):
    """The tensor-core form through the file runner keeps exactly the correlations execute() returns
    (filtered at mincorr) -- the runner and the host process() see the same device results."""
    G, S = 300, 64
    gem = synthetic.generate(3, genes=G, samples=S, seed=4)
    sim = Similarity(gem, semantics="fixed", precision=precision, mincorr=0.5)
    sim.run(cmx_path=tmp_path / "t.cmx", device_block=32768)
    res = sim.execute(None, start=0, size=sim.total_pairs())
    sim.close()
    r = res.corr[:, 0]
    keep = ~np.isnan(r) & (np.abs(r) >= np.float32(0.5)) & (np.abs(r) <= np.float32(1.0))
    x, y = pyoracle.pair_xy(np.nonzero(keep)[0])
    got = pm.read(tmp_path / "t.cmx", pm.CMX)
    assert np.array_equal(got["x"], x) and np.array_equal(got["y"], y)
    assert np.array_equal(got["payload"][:, 0], r[keep])
    assert len(x) > 0
