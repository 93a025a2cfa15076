"""CCM / CMX pairwise matrix files and EMX data (include/kinc_pairwise_matrix.h),
following the reference's round-trip tests (tests/testclustermatrix.cpp,
tests/testcorrelationmatrix.cpp, tests/testexpressionmatrix.cpp): random
contents written, read back and compared field by field.  Host code only."""
import os
import struct

import numpy as np
import pytest

from kinc_gb300 import _native, pairwise_matrix as pm


def _random_items(rng, genes, max_clusters, samples):
    xs, ys, cs, codes, corr = [], [], [], [], []
    for x in range(1, genes):
        for y in range(x):
            k = int(rng.integers(0, max_clusters + 1))
            for c in range(k):
                xs.append(x)
                ys.append(y)
                cs.append(c)
                codes.append(rng.choice([0, 1, 6, 7, 8, 9], size=samples))
                corr.append(rng.uniform(-1, 1))
    return (np.array(xs), np.array(ys), np.array(cs), np.array(codes, np.int8).reshape(-1, samples),
            np.array(corr, np.float32).reshape(-1, 1))


@pytest.mark.parametrize("little", [False, True])
def test_cluster_matrix_round_trip(tmp_path, native, little):
    rng = np.random.default_rng(1)
    genes, maxk, samples = 10, 5, 5
    x, y, c, codes, _ = _random_items(rng, genes, maxk, samples)
    path = tmp_path / "a.ccm"
    pm.write(path, pm.CCM, genes, maxk, samples, x, y, c, codes, little_endian=little)
    got = pm.read(path, pm.CCM, little_endian=little)
    assert (got["genes"], got["max_clusters"], got["subsize"]) == (genes, maxk, samples)
    assert got["pairs"] == len({(a, b) for a, b in zip(x, y)})
    assert np.array_equal(got["x"], x) and np.array_equal(got["y"], y) and np.array_equal(got["c"], c)
    assert np.array_equal(got["payload"], codes)
    # 30-byte header + 4-byte sample count + items of 9 + (5+1)/2 bytes
    assert os.path.getsize(path) == 30 + 4 + len(x) * (9 + 3)
    with open(path, "rb") as fh:
        head = fh.read(34)
    fmt = "<iiiqqhi" if little else ">iiiqqhi"
    assert struct.unpack(fmt, head) == (genes, maxk, 3, got["pairs"], len(x), 4, samples)


def test_cluster_matrix_nibbles(tmp_path, native):
    codes = np.array([[9, 1, 0, 7, 8]], np.int8)
    path = tmp_path / "n.ccm"
    pm.write(path, pm.CCM, 4, 2, 5, [3], [1], [0], codes)
    with open(path, "rb") as fh:
        raw = fh.read()
    item = raw[34:]
    assert struct.unpack(">iib", item[:9]) == (3, 1, 0)
    assert item[9:] == bytes([0x19, 0x70, 0x08])     # low nibble = even sample


@pytest.mark.parametrize("little", [False, True])
def test_correlation_matrix_round_trip(tmp_path, native, little):
    rng = np.random.default_rng(2)
    genes, maxk = 10, 5
    x, y, c, _, corr = _random_items(rng, genes, maxk, 3)
    path = tmp_path / "a.cmx"
    pm.write(path, pm.CMX, genes, maxk, 1, x, y, c, corr, little_endian=little)
    got = pm.read(path, pm.CMX, little_endian=little)
    assert np.array_equal(got["payload"], corr)
    assert np.array_equal(got["x"], x) and np.array_equal(got["c"], c)
    assert os.path.getsize(path) == 30 + 1 + len(x) * (9 + 4)


def test_wrong_byte_order_is_detected(tmp_path, native):
    path = tmp_path / "b.cmx"
    pm.write(path, pm.CMX, 5, 3, 1, [2], [0], [0], np.array([[0.7]], np.float32))
    with pytest.raises(_native.SimError):
        pm.read(path, pm.CMX, little_endian=True)


def test_order_and_index_errors(tmp_path, native):
    path = tmp_path / "c.cmx"
    with pytest.raises(_native.SimError) as e:
        pm.write(path, pm.CMX, 6, 3, 1, [3, 2], [1, 0], [0, 0], np.zeros((2, 1), np.float32))
    assert e.value.code == _native.EORDER
    with pytest.raises(_native.SimError):
        pm.write(path, pm.CMX, 6, 3, 1, [2], [2], [0], np.zeros((1, 1), np.float32))
    with pytest.raises(_native.SimError):
        pm.write(path, pm.CMX, 6, 3, 1, [2], [1], [3], np.zeros((1, 1), np.float32))
    with pytest.raises(_native.SimError):
        pm.write(path, pm.CMX, 6, 65, 1, [], [], [], np.zeros((0, 1), np.float32))


@pytest.mark.parametrize("little", [False, True])
def test_expression_matrix_round_trip(tmp_path, native, little):
    rng = np.random.default_rng(3)
    gem = rng.normal(8, 2, size=(10, 5)).astype(np.float32)
    gem[rng.random(gem.shape) < 0.2] = np.nan
    path = tmp_path / "a.emx"
    pm.write_emx(path, gem, little_endian=little)
    got = pm.read_emx(path, little_endian=little)
    assert np.array_equal(np.isnan(got), np.isnan(gem))
    assert np.array_equal(got[~np.isnan(gem)], gem[~np.isnan(gem)])
    assert os.path.getsize(path) == 8 + gem.size * 4


def test_truncated_expression_matrix(tmp_path, native):
    path = tmp_path / "t.emx"
    with open(path, "wb") as fh:
        fh.write(struct.pack(">ii", 10, 5) + b"\0" * 12)
    with pytest.raises(_native.SimError, match="truncated"):
        pm.read_emx(path)
    with open(path, "wb") as fh:
        fh.write(b"\0\0")
    with pytest.raises(_native.SimError, match="truncated EMX header"):
        pm.read_emx(path)


@pytest.mark.parametrize("little", [False, True])
def test_export_text_matches_restatement(tmp_path, native, little):
    """kinc_pm_export_text equals ExportCorrelationMatrix::process restated over the same files:
    CCM data only for pairs with more than one CMX cluster, first correlation at %.6g."""
    from oracle import pyoracle
    rng = np.random.default_rng(7)
    genes, maxk, samples = 12, 4, 9
    xs, ys, cs, codes, corr = [], [], [], [], []
    mx, my, mc, mcodes = [], [], [], []
    specials = [1e-5, -0.0, 0.5, 1.0, -0.999999, 123456.7, 3.0e-7]
    for x in range(1, genes):
        for y in range(x):
            k = int(rng.integers(0, maxk + 1))
            in_ccm = k > 1 or (k == 1 and rng.random() < 0.5)   # a K > 1 pair with one kept cluster
            for c in range(k):
                xs.append(x)
                ys.append(y)
                cs.append(c)
                r0 = specials[len(corr) % len(specials)] if rng.random() < 0.2 else rng.uniform(-1, 1)
                corr.append([r0, rng.uniform(-1, 1)])
                if in_ccm:
                    mx.append(x)
                    my.append(y)
                    mc.append(c)
                    mcodes.append(rng.choice([0, 1, 6, 7, 8, 9], size=samples))
    corr = np.array(corr, np.float32)
    ccm_path, cmx_path, out = tmp_path / "e.ccm", tmp_path / "e.cmx", tmp_path / "e.txt"
    pm.write(cmx_path, pm.CMX, genes, maxk, 2, xs, ys, cs, corr, little_endian=little)
    pm.write(ccm_path, pm.CCM, genes, maxk, samples, mx, my, mc, np.array(mcodes, np.int8).reshape(-1, samples),
             little_endian=little)
    pm.export_text(ccm_path, cmx_path, out, little_endian=little)
    want = pyoracle.export_text(pm.read(cmx_path, pm.CMX, little_endian=little),
                                pm.read(ccm_path, pm.CCM, little_endian=little), samples)
    got = out.read_text()
    assert got == want
    assert len(got.splitlines()) == len(xs)
    assert "\t1e-05\t" in got or "\t-0\t" in got or "\t0.5\t" in got


def test_export_text_rejects_missing_ccm_pair(tmp_path, native):
    """A CMX pair with several clusters needs its CCM clusters (the reference would read past them)."""
    pm.write(tmp_path / "m.cmx", pm.CMX, 5, 3, 1, [2, 2], [1, 1], [0, 1], np.array([[0.9], [0.8]], np.float32))
    pm.write(tmp_path / "m.ccm", pm.CCM, 5, 3, 4, [3], [0], [0], np.zeros((1, 4), np.int8))
    with pytest.raises(_native.SimError):
        pm.export_text(tmp_path / "m.ccm", tmp_path / "m.cmx", tmp_path / "m.txt")


@pytest.mark.parametrize("named", [False, True])
def test_extract_matches_restatement(tmp_path, native, named):
    """kinc_pm_extract writes the TSV edge list and the GraphML that Extract::process restated
    writes from the same EMX/CCM/CMX: threshold on the first correlation, CCM counts and mask for
    multi-cluster pairs, EMX missing-value mask for single-cluster pairs."""
    from oracle import pyoracle
    rng = np.random.default_rng(11)
    genes, maxk, samples = 14, 4, 10
    gem = (8 + 2 * rng.standard_normal((genes, samples))).astype(np.float32)
    gem[rng.random(gem.shape) < 0.2] = np.nan
    xs, ys, cs, corr, mx, my, mc, mcodes = [], [], [], [], [], [], [], []
    for x in range(1, genes):
        for y in range(x):
            k = int(rng.integers(0, maxk + 1))
            for c in range(k):
                xs.append(x); ys.append(y); cs.append(c)
                corr.append([rng.choice([0.85, -0.85, 0.9, -0.99, 1.0, 0.5, 0.84999996]), rng.uniform(-1, 1)])
                if k > 1:
                    mx.append(x); my.append(y); mc.append(c)
                    mcodes.append(rng.choice([0, 1, 6, 7, 8, 9], size=samples))
    corr = np.array(corr, np.float32)
    emx, ccm_path, cmx_path = tmp_path / "g.emx", tmp_path / "g.ccm", tmp_path / "g.cmx"
    pm.write_emx(emx, gem)
    pm.write(cmx_path, pm.CMX, genes, maxk, 2, xs, ys, cs, corr)
    pm.write(ccm_path, pm.CCM, genes, maxk, samples, mx, my, mc, np.array(mcodes, np.int8).reshape(-1, samples))
    names = [f"gene_{g:03d}" for g in range(genes)] if named else None
    names_path = None
    if named:
        names_path = tmp_path / "names.txt"
        names_path.write_text("\n".join(names) + "\n")
    pm.extract(emx, ccm_path, cmx_path, tsv_path=tmp_path / "n.tsv", graphml_path=tmp_path / "n.graphml",
               names_path=names_path)
    want_tsv, want_gml = pyoracle.extract_network(gem, pm.read(cmx_path, pm.CMX), pm.read(ccm_path, pm.CCM), samples,
                                                  names=names)
    assert (tmp_path / "n.tsv").read_text() == want_tsv
    assert (tmp_path / "n.graphml").read_text() == want_gml
    assert want_tsv.count("\n") > 5


def test_export_text_literal_lines(tmp_path, native):
    """Exact text for a small case written out by hand from ExportCorrelationMatrix::process
    (src/core/exportcorrelationmatrix.cpp:44-100): counts of codes 1, 9, 8, 7, 6 in that column
    order, the first correlation at precision 6, the mask '0' + code; a single-cluster pair gets
    zero counts and an all-'0' mask even when the CCM holds its cluster."""
    pm.write(tmp_path / "l.cmx", pm.CMX, 5, 3, 2, [2, 2, 4], [0, 0, 3], [0, 1, 0],
             np.array([[0.123456789, 9.0], [-1.0, 9.0], [0.5, 9.0]], np.float32))
    pm.write(tmp_path / "l.ccm", pm.CCM, 5, 3, 6, [2, 2, 4], [0, 0, 3], [0, 1, 0],
             np.array([[1, 1, 9, 8, 7, 6], [0, 0, 1, 1, 1, 9], [1, 1, 1, 1, 1, 1]], np.int8))
    pm.export_text(tmp_path / "l.ccm", tmp_path / "l.cmx", tmp_path / "l.txt")
    assert (tmp_path / "l.txt").read_text().splitlines() == [
        "2\t0\t0\t2\t2\t1\t1\t1\t1\t0.123457\t119876",
        "2\t0\t1\t2\t3\t1\t0\t0\t0\t-1\t001119",
        "4\t3\t0\t1\t0\t0\t0\t0\t0\t0.5\t000000",
    ]


def test_extract_literal_lines(tmp_path, native):
    """Exact TSV and GraphML for a small case written out by hand from Extract::process
    (src/core/extract.cpp:24-274): the header line, |r| >= mincorr only, single-cluster masks from
    the expression matrix ('9' where either gene is NaN)."""
    gem = np.array([[1, 2, np.nan, 4], [1, 2, 3, 4], [1, np.nan, 3, 4]], np.float32)
    pm.write_emx(tmp_path / "e.emx", gem)
    pm.write(tmp_path / "e.cmx", pm.CMX, 3, 2, 1, [1, 2, 2], [0, 1, 1], [0, 0, 1],
             np.array([[0.9], [0.95], [0.2]], np.float32))
    pm.write(tmp_path / "e.ccm", pm.CCM, 3, 2, 4, [2, 2], [1, 1], [0, 1],
             np.array([[1, 9, 1, 7], [0, 9, 0, 1]], np.int8))
    pm.extract(tmp_path / "e.emx", tmp_path / "e.ccm", tmp_path / "e.cmx", tsv_path=tmp_path / "e.tsv",
               graphml_path=tmp_path / "e.graphml", min_corr=0.85)
    assert (tmp_path / "e.tsv").read_text().splitlines() == [
        "Source\tTarget\tsc\tInteraction\tCluster\tNum_Clusters\tCluster_Samples\tMissing_Samples\t"
        "Cluster_Outliers\tPair_Outliers\tToo_Low\tSamples",
        "1\t0\t0.9\tco\t0\t1\t0\t0\t0\t0\t0\t1191",
        "2\t1\t0.95\tco\t0\t2\t2\t1\t0\t1\t0\t1917",
    ]
    g = (tmp_path / "e.graphml").read_text()
    assert g.count('<node id="') == 3
    assert '<edge source="1" target="0" samples="1191"/>' in g
    assert '<edge source="2" target="1" samples="1917"/>' in g
    assert g.endswith("  </graph>\n</graphml>\n")


def test_unwritable_output_is_an_io_error(tmp_path, native):
    """A file that cannot be written reports KINC_SIM_EIO (or EINVAL when it cannot even be opened)."""
    import os
    if os.geteuid() == 0:
        target = "/proc/self/does-not-exist/x.cmx"     # root can write anywhere else
    else:
        d = tmp_path / "ro"
        d.mkdir()
        os.chmod(d, 0o500)
        target = str(d / "x.cmx")
    with pytest.raises(_native.SimError) as err:
        pm.write(target, pm.CMX, 4, 2, 1, [1], [0], [0], np.array([[0.5]], np.float32))
    assert err.value.code in (_native.EINVAL, _native.EIO)


@pytest.mark.parametrize("little", [False, True])
@pytest.mark.parametrize("kind", ["ccm", "cmx"])
def test_concat_rejoins_split_files(tmp_path, native, little, kind):
    """A file cut into three item ranges (one cut inside a pair's clusters) and joined again is
    byte for byte the original; the header counts are recomputed."""
    rng = np.random.default_rng(6)
    genes, maxk, samples = 14, 4, 9
    x, y, c, codes, corr = _random_items(rng, genes, maxk, samples)
    t = pm.CCM if kind == "ccm" else pm.CMX
    payload = codes if kind == "ccm" else corr
    sub = samples if kind == "ccm" else 1
    pm.write(tmp_path / f"a.{kind}", t, genes, maxk, sub, x, y, c, payload, little_endian=little)
    multi = [i for i in range(1, len(x)) if (x[i], y[i]) == (x[i - 1], y[i - 1])]
    cuts = [0, multi[len(multi) // 2], 2 * len(x) // 3, len(x)]
    parts = []
    for k in range(3):
        sl = slice(cuts[k], cuts[k + 1])
        parts.append(tmp_path / f"p{k}.{kind}")
        pm.write(parts[-1], t, genes, maxk, sub, x[sl], y[sl], c[sl], payload[sl], little_endian=little)
    pm.concat(tmp_path / f"b.{kind}", parts, little_endian=little)
    assert (tmp_path / f"b.{kind}").read_bytes() == (tmp_path / f"a.{kind}").read_bytes()


def test_concat_errors(tmp_path, native):
    rng = np.random.default_rng(7)
    x, y, c, codes, corr = _random_items(rng, 10, 3, 5)
    pm.write(tmp_path / "a.cmx", pm.CMX, 10, 3, 1, x, y, c, corr)
    pm.write(tmp_path / "b.cmx", pm.CMX, 11, 3, 1, x, y, c, corr)
    pm.write(tmp_path / "a.ccm", pm.CCM, 10, 3, 5, x, y, c, codes)
    with pytest.raises(_native.SimError, match="does not match"):
        pm.concat(tmp_path / "o.cmx", [tmp_path / "a.cmx", tmp_path / "b.cmx"])
    assert not (tmp_path / "o.cmx").exists()
    with pytest.raises(_native.SimError) as e:      # the same items twice: out of order at the join
        pm.concat(tmp_path / "o.cmx", [tmp_path / "a.cmx", tmp_path / "a.cmx"])
    assert e.value.code == _native.EORDER
    with pytest.raises(_native.SimError, match="not a CMX"):     # a CCM among CMX files
        pm.concat(tmp_path / "o.cmx", [tmp_path / "a.cmx", tmp_path / "a.ccm"])
    with pytest.raises(_native.SimError, match="is also input"):
        pm.concat(tmp_path / "a.cmx", [tmp_path / "a.cmx"])
    assert pm.read(tmp_path / "a.cmx", pm.CMX)["x"].size == len(x)    # the input was left alone


def _blocks_of_items(rng, genes, samples, maxk=3):
    """CMX items for every pair (1..maxk clusters), CCM items for the multi-cluster pairs."""
    xs, ys = np.tril_indices(genes, -1)
    k = rng.integers(1, maxk + 1, size=len(xs))
    X, Y = np.repeat(xs, k).astype(np.int32), np.repeat(ys, k).astype(np.int32)
    C = np.concatenate([np.arange(kk) for kk in k]).astype(np.int8)
    R = rng.uniform(-1, 1, (len(X), 1)).astype(np.float32)
    multi = np.repeat(k, k) > 1
    codes = rng.choice(np.array([0, 1, 6, 7, 8, 9], np.int8), size=(int(multi.sum()), samples))
    return (X, Y, C, R), (X[multi], Y[multi], C[multi], codes)


@pytest.mark.parametrize("little", [False, True])
def test_resume_point_cuts_back_to_whole_blocks(tmp_path, native, little):
    """An interrupted run (header counts still those of a new file, the last item cut short):
    the files are cut back to the work blocks before the one holding the last whole item, and
    the rest of the run joined after them gives the files of the uninterrupted run."""
    rng = np.random.default_rng(8)
    genes, samples, maxk = 450, 6, 3                 # 100,925 pairs: four work blocks
    cmx, ccm = _blocks_of_items(rng, genes, samples, maxk)
    full = {}
    for kind, items, t, sub in (("cmx", cmx, pm.CMX, 1), ("ccm", ccm, pm.CCM, samples)):
        pm.write(tmp_path / f"full.{kind}", t, genes, maxk, sub, *items, little_endian=little)
        full[kind] = (tmp_path / f"full.{kind}").read_bytes()
    B = 32768
    # interrupt: CMX written up to the middle of block 2 (plus half an item), CCM to block 1
    for kind, items, cut_pair, sub in (("cmx", cmx, 2 * B + 5000, 1), ("ccm", ccm, B + 700, samples)):
        x, y = items[0].astype(np.int64), items[1].astype(np.int64)
        n_keep = int(np.searchsorted(x * (x - 1) // 2 + y, cut_pair))
        head = 30 + (1 if kind == "cmx" else 4)
        item = 9 + (4 if kind == "cmx" else (samples + 1) // 2)
        raw = bytearray(full[kind][:head + n_keep * item + item // 2])
        raw[12:28] = bytes(16)                          # counts as kinc_pm_create wrote them
        (tmp_path / f"run.{kind}").write_bytes(bytes(raw))
    R = pm.resume_point(tmp_path / "run.ccm", tmp_path / "run.cmx", little_endian=little)
    assert R == 1                                       # the CCM's last whole item is in block 1
    for kind, items, t, sub in (("cmx", cmx, pm.CMX, 1), ("ccm", ccm, pm.CCM, samples)):
        x, y = items[0].astype(np.int64), items[1].astype(np.int64)
        keep = (x * (x - 1) // 2 + y) < R * B
        pm.write(tmp_path / f"want.{kind}", t, genes, maxk, sub, *[a[keep] for a in items], little_endian=little)
        assert (tmp_path / f"run.{kind}").read_bytes() == (tmp_path / f"want.{kind}").read_bytes(), kind
        pm.write(tmp_path / f"part.{kind}", t, genes, maxk, sub, *[a[~keep] for a in items], little_endian=little)
        pm.concat(tmp_path / f"joined.{kind}", [tmp_path / f"run.{kind}", tmp_path / f"part.{kind}"],
                  little_endian=little)
        assert (tmp_path / f"joined.{kind}").read_bytes() == full[kind], kind


def test_resume_point_edge_cases(tmp_path, native):
    # no files yet: start at the shard's first block
    assert pm.resume_point(tmp_path / "none.ccm", tmp_path / "none.cmx", first_block=5) == 5
    # a file without items, the other file not written
    pm.write(tmp_path / "e.cmx", pm.CMX, 10, 2, 1, [], [], [], np.zeros((0, 1), np.float32))
    assert pm.resume_point(None, tmp_path / "e.cmx", first_block=3) == 3
    # a file not created yet: everything runs again, the other file is cut back to the start
    pm.write(tmp_path / "f.cmx", pm.CMX, 10, 2, 1, [3, 5], [1, 2], [0, 0], np.array([[0.5], [0.6]], np.float32))
    assert pm.resume_point(tmp_path / "missing.ccm", tmp_path / "f.cmx", first_block=0) == 0
    assert pm.read(tmp_path / "f.cmx", pm.CMX)["x"].size == 0
    # items of blocks below the shard's first block are never the resume point
    pm.write(tmp_path / "s.cmx", pm.CMX, 10, 2, 1, [3], [1], [0], np.array([[0.5]], np.float32))
    assert pm.resume_point(None, tmp_path / "s.cmx", first_block=2) == 2
    assert pm.read(tmp_path / "s.cmx", pm.CMX)["x"].size == 1
    with pytest.raises(_native.SimError, match="not a CCM"):
        pm.resume_point(tmp_path / "s.cmx", None)
