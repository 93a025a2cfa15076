"""Host-side mirror of the Similarity analytic: arguments, block split and
the ordered pairwise-matrix writer (no GPU)."""
import math

import numpy as np
import pytest

from kinc_gb300 import InvalidArgument, PairwiseMatrix, Similarity


def test_defaults_and_choices():
    s = Similarity(np.zeros((10, 5), np.float32))
    p = s.params
    assert (p.clus_method, p.corr_method, p.criterion, p.min_samples) == (0, 0, 1, 30)
    assert math.isinf(p.min_expr) and p.min_expr < 0
    s = Similarity(np.zeros((10, 5), np.float32), clusmethod="gmm", corrmethod="spearman", crit="BIC")
    assert (s.params.clus_method, s.params.corr_method, s.params.criterion) == (1, 1, 0)
    with pytest.raises(InvalidArgument):
        Similarity(np.zeros((10, 5), np.float32), clusmethod="dbscan")


@pytest.mark.parametrize("name,value", [("fp32", 0), ("tf32", 1), ("3xbf16", 2), ("fp32tiled", 3), ("fp16", 4)])
def test_precision_names_map_to_the_abi(name, value):
    """The precision names of the Python mirror and the CLI, and the ABI's kinc_sim_params.precision."""
    s = Similarity(np.zeros((10, 5), np.float32), semantics="fixed", precision=name)
    assert s.params.precision == value


def test_unknown_precision_is_rejected():
    with pytest.raises(InvalidArgument):
        Similarity(np.zeros((10, 5), np.float32), precision="fp8")


def test_cluster_range_check():
    s = Similarity(np.zeros((10, 5), np.float32), minclus=4, maxclus=2)
    with pytest.raises(InvalidArgument, match="Minimum clusters"):
        s.initialize()


@pytest.mark.parametrize("genes", [2, 3, 257, 1000, 30000])
def test_block_split(genes):
    s = Similarity(np.zeros((genes, 1), np.float32))
    total = genes * (genes - 1) // 2
    assert s.size() == (total + 32767) // 32768
    blocks = [s.make_work(i) for i in range(s.size())]
    assert blocks[0].start == 0
    assert sum(b.size for b in blocks) == total
    assert all(b.size == 32768 for b in blocks[:-1])


def test_pairwise_matrix_order_is_enforced():
    m = PairwiseMatrix("cmx", 10, 5, 4)
    m.write_pair(1, 0, [0.9])
    m.write_pair(2, 1, [0.5, -0.7])
    with pytest.raises(ValueError, match="Attempting to write indent"):
        m.write_pair(2, 0, [0.8])
    with pytest.raises(ValueError, match="exceeding the max"):
        m.write_pair(9, 8, [0.1] * 6)
    x, y, c, r = m.arrays()
    assert list(c) == [0, 0, 1] and m.pairs == 2


def test_resume_runs_only_the_missing_blocks(tmp_path, native, monkeypatch):
    """Similarity.run(resume=True) on files an interrupted run left: they are cut back to whole
    work blocks, only the blocks from there on run again (into part files), and the joined files
    equal those of the uninterrupted run.  The worker is replaced by a deterministic item
    generator, so this checks the orchestration on the CPU."""
    import numpy as np

    from kinc_gb300 import Similarity, pairwise_matrix as pm
    B, S, maxk = 32768, 8, 3
    gem = np.zeros((450, S), np.float32)                 # 100,925 pairs: four work blocks
    G = gem.shape[0]
    total = G * (G - 1) // 2
    ran = []

    def fake_run(self, ccm, cmx, le, first, n, dev):
        if n < 0:                                        # the runner's "all remaining blocks"
            n = -(-total // B) - first
        ran.append((first, n))
        lo, hi = first * B, min(total, (first + n) * B)
        p = np.arange(lo, hi, dtype=np.int64)
        x = np.floor((1 + np.sqrt(1 + 8 * p.astype(np.float64))) / 2).astype(np.int64)
        x -= (x * (x - 1) // 2 > p)
        y = p - x * (x - 1) // 2
        k = (p * 7919) % (maxk + 1)
        X, Y = np.repeat(x, k), np.repeat(y, k)
        C = np.concatenate([np.arange(kk) for kk in k]) if len(k) else np.zeros(0, np.int64)
        R = ((np.repeat(p, k) % 1000) / 1000.0).astype(np.float32).reshape(-1, 1)
        m = np.repeat(k, k) > 1
        codes = (np.repeat(p, k)[m][:, None] + np.arange(S)[None, :]) % 2
        if cmx is not None:
            pm.write(cmx, pm.CMX, G, maxk, 1, X, Y, C, R, little_endian=le)
        if ccm is not None:
            pm.write(ccm, pm.CCM, G, maxk, S, X[m], Y[m], C[m], codes.astype(np.int8), little_endian=le)

    monkeypatch.setattr(Similarity, "_run_to_files", fake_run)
    sim = Similarity(gem, clusmethod="gmm", maxclus=maxk)
    sim.run(ccm_path=tmp_path / "full.ccm", cmx_path=tmp_path / "full.cmx")
    full = {e: (tmp_path / f"full.{e}").read_bytes() for e in ("ccm", "cmx")}
    # the interrupted run: both files cut inside block 2 (CMX further than CCM), counts as at creation
    for e, cut in (("cmx", 0.9), ("ccm", 0.7)):
        raw = bytearray(full[e][:int(len(full[e]) * cut)])
        raw[12:28] = bytes(16)
        (tmp_path / f"run.{e}").write_bytes(bytes(raw))
    ran.clear()
    sim.run(ccm_path=tmp_path / "run.ccm", cmx_path=tmp_path / "run.cmx", resume=True)
    assert ran == [(2, 2)]                               # blocks 2 and 3 only
    for e in ("ccm", "cmx"):
        assert (tmp_path / f"run.{e}").read_bytes() == full[e], e
        assert not (tmp_path / f"run.{e}.part").exists()
    # a rank's share: the interrupted files of rank 1 of 2 resume inside its own range
    sim.run(ccm_path=tmp_path / "r1.ccm", cmx_path=tmp_path / "r1.cmx", world=2, rank=1)
    r1 = (tmp_path / "r1.cmx").read_bytes()
    (tmp_path / "r1.cmx").write_bytes(r1[:len(r1) // 2])
    ran.clear()
    sim.run(ccm_path=tmp_path / "r1.ccm", cmx_path=tmp_path / "r1.cmx", world=2, rank=1, resume=True)
    assert ran[0][0] >= 2 and ran[0][0] + ran[0][1] == 4
    assert (tmp_path / "r1.cmx").read_bytes() == r1
