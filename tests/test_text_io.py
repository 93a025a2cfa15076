"""The text analytics around the matrix files (include/kinc_pairwise_matrix.h): import-cmx
(ImportCorrelationMatrix), import-emx and export-emx (ImportExpressionMatrix,
ExportExpressionMatrix), checked against the oracle's restatements of the reference's
code, through round trips, and on the reference's error cases.  Host code only."""
import math
import subprocess

import numpy as np
import pytest

from kinc_gb300 import _native, build, pairwise_matrix as pm
from kinc_gb300 import __main__ as cli
from oracle import pyoracle


def _similarity_like_items(rng, genes, maxk, samples):
    """Items as a Similarity run writes them: every pair with 0..maxk clusters, CCM rows only for
    pairs with more than one cluster, cluster codes 0/1/6/7/8/9."""
    cmx, ccm = dict(x=[], y=[], c=[], r=[]), dict(x=[], y=[], c=[], codes=[])
    for x in range(1, genes):
        for y in range(x):
            k = int(rng.integers(0, maxk + 1))
            for c in range(k):
                cmx["x"].append(x), cmx["y"].append(y), cmx["c"].append(c)
                cmx["r"].append([rng.uniform(-1, 1)])
                if k > 1:
                    ccm["x"].append(x), ccm["y"].append(y), ccm["c"].append(c)
                    ccm["codes"].append(rng.choice([0, 1, 6, 7, 8, 9], size=samples))
    return cmx, ccm


def _write_pair_files(tmp_path, rng, genes=12, maxk=3, samples=7, little=False):
    cmx, ccm = _similarity_like_items(rng, genes, maxk, samples)
    pm.write(tmp_path / "a.cmx", pm.CMX, genes, maxk, 1, cmx["x"], cmx["y"], cmx["c"],
             np.array(cmx["r"], np.float32), little_endian=little)
    pm.write(tmp_path / "a.ccm", pm.CCM, genes, maxk, samples, ccm["x"], ccm["y"], ccm["c"],
             np.array(ccm["codes"], np.int8).reshape(-1, samples), little_endian=little)
    return genes, maxk, samples


@pytest.mark.parametrize("little", [False, True])
def test_import_cmx_reads_back_what_export_writes(tmp_path, native, little):
    genes, maxk, samples = _write_pair_files(tmp_path, np.random.default_rng(3), little=little)
    pm.export_text(tmp_path / "a.ccm", tmp_path / "a.cmx", tmp_path / "a.txt", little_endian=little)
    pm.import_text(tmp_path / "a.txt", tmp_path / "b.ccm", tmp_path / "b.cmx", genes, maxk, samples,
                   little_endian=little)
    # the cluster matrix comes back byte for byte (header counts included)
    assert (tmp_path / "b.ccm").read_bytes() == (tmp_path / "a.ccm").read_bytes()
    a = pm.read(tmp_path / "a.cmx", pm.CMX, little_endian=little)
    b = pm.read(tmp_path / "b.cmx", pm.CMX, little_endian=little)
    for key in ("genes", "max_clusters", "subsize", "pairs"):
        assert a[key] == b[key]
    for key in ("x", "y", "c"):
        assert np.array_equal(a[key], b[key])
    # correlations were written at 6 significant digits
    want = np.array([np.float32(float("%.6g" % float(r))) for r in a["payload"][:, 0]], np.float32)
    assert np.array_equal(b["payload"][:, 0], want)
    # and exporting the imported files gives the same text
    pm.export_text(tmp_path / "b.ccm", tmp_path / "b.cmx", tmp_path / "b.txt", little_endian=little)
    assert (tmp_path / "b.txt").read_text() == (tmp_path / "a.txt").read_text()


def test_import_cmx_matches_restatement(tmp_path, native):
    S = 6
    text = ("#\n"                                           # a one-field marker line
            "\n"
            "3\t1\t0\t1\t5\t0\t0\t0\t0\t0.912345678\t000000\n"
            "  5 2 0 2 2 1 1 1 1 -0.95 119780\r\n"            # spaces and CRLF
            "5\t2\t1\t2\t0\t0\t0\t0\t0\t1e-1\t0a1b1c\n"       # non-digit mask characters: code 15
            "7 0 0 1 0 0 0 0 0 abc 111111\n"                   # a correlation that is not a number reads 0
            "8 6 9 9 9 9 9 9 9 +0.5 999999\n"
            "8 6 9 9 9 9 9 9 9 -inf 000000\n"
            "8 6 9 9 9 9 9 9 9 .25 161616\n"
            "x\n")
    (tmp_path / "t.txt").write_text(text)
    pm.import_text(tmp_path / "t.txt", tmp_path / "t.ccm", tmp_path / "t.cmx", 9, 3, S)
    ccm, cmx = pyoracle.import_cmx_text(text, 9, 3, S)
    got_ccm = pm.read(tmp_path / "t.ccm", pm.CCM)
    got_cmx = pm.read(tmp_path / "t.cmx", pm.CMX)
    for want, got in ((ccm, got_ccm), (cmx, got_cmx)):
        for key in ("x", "y", "c"):
            assert np.array_equal(got[key], want[key]), key
    assert np.array_equal(got_cmx["payload"].view(np.uint32), cmx["payload"].view(np.uint32))
    # CCM codes are stored as nibbles: the -1 of a non-digit mask character reads back as 15
    assert np.array_equal(got_ccm["payload"] & 0x0F, ccm["payload"] & 0x0F)
    assert (got_cmx["pairs"], got_ccm["pairs"]) == (4, 2)
    assert list(got_cmx["payload"][:, 0][[0, 3]]) == [np.float32(0.912345678), np.float32(0.0)]


@pytest.mark.parametrize("line,code,msg", [
    ("3 1 0 1 0 0 0 0 0 0.9", _native.EINVAL, "incorrect amount of fields"),
    ("3 1 0 1 0 0 0 0 0 0.9 0000", _native.EINVAL, "invalid length 4"),
    ("1 3 0 1 0 0 0 0 0 0.9 00000", _native.EINVAL, "Cannot initialize pairwise index"),
    ("9 3 0 1 0 0 0 0 0 0.9 00000", _native.EINVAL, "Cannot initialize pairwise index"),
    ("2 0 0 1 0 0 0 0 0 0.9 00000", _native.EORDER, "Attempting to write indent"),
    ("4 2 0 1 0 0 0 0 0 0.9 00000\n4 2 0 1 0 0 0 0 0 0.9 00000", _native.EINVAL, "exceeding the max of 2"),
])
def test_import_cmx_errors(tmp_path, native, line, code, msg):
    """The reference's parse errors, and Matrix::write's order and cluster-count rules."""
    text = "4 2 0 1 0 0 0 0 0 0.9 00000\n" + line + "\n"
    (tmp_path / "t.txt").write_text(text)
    with pytest.raises(_native.SimError) as e:
        pm.import_text(tmp_path / "t.txt", tmp_path / "t.ccm", tmp_path / "t.cmx", 8, 2, 5)
    assert e.value.code == code and msg in str(e.value)
    assert f"(line {2 + line.count(chr(10))})" in str(e.value)
    with pytest.raises(pyoracle.TextError):
        pyoracle.import_cmx_text(text, 8, 2, 5)


def _gem_text(rng, genes, samples, nan="NA", header=True, positive=False):
    """Expression text in the number spellings Qt's toDouble reads."""
    spell = [lambda v: "%.9g" % v, lambda v: "%.3e" % v, lambda v: "%+.4f" % v, lambda v: "%.17g" % v]
    lines = ["\t".join(f"s{i}" for i in range(samples)) + "\t"] if header else []
    for g in range(genes):
        vals = []
        for s in range(samples):
            if rng.random() < 0.1:
                vals.append(nan)
            else:
                v = float(rng.uniform(0.01, 20) if positive else rng.normal(8, 4))
                vals.append(spell[int(rng.integers(0, len(spell)))](v))
        lines.append(f"gene_{g} " + " ".join(vals))
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("transform", [0, 1, 2, 3])
@pytest.mark.parametrize("header", [True, False])
def test_import_emx_matches_restatement(tmp_path, native, transform, header):
    rng = np.random.default_rng(10 + transform)
    G, S = 40, 13
    text = _gem_text(rng, G, S, header=header, positive=transform != 0)
    (tmp_path / "g.txt").write_text(text)
    pm.import_emx_text(tmp_path / "g.txt", tmp_path / "g.emx", nan="NA", samples=0 if header else S,
                       transform=pm.TRANSFORMS[transform], gene_names_path=tmp_path / "genes",
                       sample_names_path=tmp_path / "samples")
    gem, genes, samples = pyoracle.import_emx_text(text, nan="NA", samples=0 if header else S, transform=transform)
    got = pm.read_emx(tmp_path / "g.emx")
    assert got.shape == (G, S)
    assert np.array_equal(got.view(np.uint32), gem.view(np.uint32))
    assert (tmp_path / "genes").read_text().split("\n")[:-1] == genes == [f"gene_{g}" for g in range(G)]
    want_samples = [f"s{i}" for i in range(S)] if header else [str(i) for i in range(S)]
    assert (tmp_path / "samples").read_text().split("\n")[:-1] == samples == want_samples


def test_import_emx_number_spellings(tmp_path, native):
    text = "a b c d e f g h\ng1 1 +2.5 -.5 1e3 1E-3 inf -inf 7.\ng2 nan 0 -0 3.25e+2 NA 1.5 2 3\n"
    (tmp_path / "g.txt").write_text(text)
    pm.import_emx_text(tmp_path / "g.txt", tmp_path / "g.emx", nan="NA")
    got = pm.read_emx(tmp_path / "g.emx")
    want = np.array([[1, 2.5, -0.5, 1000, 0.001, math.inf, -math.inf, 7],
                     [math.nan, 0, -0.0, 325, math.nan, 1.5, 2, 3]], np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    gem, _, _ = pyoracle.import_emx_text(text, nan="NA")
    assert np.array_equal(got.view(np.uint32), gem.view(np.uint32))


@pytest.mark.parametrize("text,msg", [
    ("a b c\ng1 1 2\n", "Read in 2 fields when it should have been 3. Gene name is g1."),
    ("a b\ng1 1 x\n", 'Failed to read expression value "x" for gene g1.'),
    ("a b\ng1 1 0x10\n", 'Failed to read expression value "0x10"'),
    ("a b\ng1 1 1e400\n", 'Failed to read expression value "1e400"'),
    ("a b\ng1 1 -nan\n", 'Failed to read expression value "-nan"'),
    ("a b\n", "holds no genes"),
])
def test_import_emx_errors(tmp_path, native, text, msg):
    (tmp_path / "g.txt").write_text(text)
    with pytest.raises(_native.SimError) as e:
        pm.import_emx_text(tmp_path / "g.txt", tmp_path / "g.emx")
    assert e.value.code == _native.EINVAL and msg in str(e.value)
    if "no genes" not in msg:
        with pytest.raises(pyoracle.TextError):
            pyoracle.import_emx_text(text)


@pytest.mark.parametrize("transform", [0, 1, 2, 3])
def test_export_emx_matches_restatement(tmp_path, native, transform):
    rng = np.random.default_rng(20 + transform)
    gem = rng.normal(2, 1.5, (30, 11)).astype(np.float32)
    gem[rng.random(gem.shape) < 0.1] = np.nan
    gem[0, 0], gem[0, 1], gem[0, 2], gem[0, 3] = np.float32(1e-30), np.float32(-3.4e38), np.inf, -np.inf
    pm.write_emx(tmp_path / "g.emx", gem)
    (tmp_path / "genes").write_text("".join(f"G{g}\n" for g in range(30)))
    pm.export_emx_text(tmp_path / "g.emx", tmp_path / "g.txt", nan="NA", transform=transform,
                       gene_names_path=tmp_path / "genes")
    want = pyoracle.export_emx_text(gem, gene_names=[f"G{g}" for g in range(30)], transform=transform, nan="NA")
    assert (tmp_path / "g.txt").read_text() == want


def test_export_emx_layout(tmp_path, native):
    gem = np.array([[1.5, np.nan], [0.1, -2.0]], np.float32)
    pm.write_emx(tmp_path / "g.emx", gem)
    pm.export_emx_text(tmp_path / "g.emx", tmp_path / "g.txt")
    # sample names each followed by a tab; a missing value is the (empty) token; 12 significant digits
    assert (tmp_path / "g.txt").read_text() == "0\t1\t\n0\t1.5\t\n1\t0.10000000149\t-2\n"


@pytest.mark.parametrize("little", [False, True])
def test_emx_text_round_trip(tmp_path, native, little):
    """export-emx then import-emx gives the matrix back bit for bit (12 digits hold a float)."""
    rng = np.random.default_rng(5)
    gem = (rng.standard_normal((50, 17)) * 10 ** rng.uniform(-8, 8, (50, 17))).astype(np.float32)
    gem[rng.random(gem.shape) < 0.05] = np.nan
    pm.write_emx(tmp_path / "a.emx", gem, little_endian=little)
    pm.export_emx_text(tmp_path / "a.emx", tmp_path / "a.txt", nan="NA", little_endian=little)
    pm.import_emx_text(tmp_path / "a.txt", tmp_path / "b.emx", nan="NA", little_endian=little)
    assert (tmp_path / "b.emx").read_bytes() == (tmp_path / "a.emx").read_bytes()


def test_names_files_must_match_the_matrix(tmp_path, native):
    pm.write_emx(tmp_path / "g.emx", np.zeros((3, 2), np.float32))
    (tmp_path / "genes").write_text("a\nb\n")
    with pytest.raises(_native.SimError, match="holds 2 names for 3 genes"):
        pm.export_emx_text(tmp_path / "g.emx", tmp_path / "g.txt", gene_names_path=tmp_path / "genes")
    with pytest.raises(ValueError):
        pm.export_emx_text(tmp_path / "g.emx", tmp_path / "g.txt", transform="log")


def test_command_lines_convert_text(tmp_path, native):
    """python -m kinc_gb300 and the native program: import-emx -> export-emx, and
    export-cmx -> import-cmx, writing the same files."""
    rng = np.random.default_rng(9)
    text = _gem_text(rng, 20, 6)
    (tmp_path / "g.txt").write_text(text)
    exe = build.CLI
    runs = {
        "py": lambda *a: cli.main(list(a)),
        "native": lambda *a: subprocess.run([exe, *a], capture_output=True, text=True).returncode,
    }
    for tag, run in runs.items():
        assert run("run", "import-emx", "--input", str(tmp_path / "g.txt"), "--output", str(tmp_path / f"{tag}.emx"),
                   "--nan", "NA", "--names", str(tmp_path / f"{tag}.genes"),
                   "--sample-names", str(tmp_path / f"{tag}.samples")) == 0
        assert run("run", "export-emx", "--input", str(tmp_path / f"{tag}.emx"), "--output",
                   str(tmp_path / f"{tag}.txt"), "--nan", "NA", "--names", str(tmp_path / f"{tag}.genes"),
                   "--sample-names", str(tmp_path / f"{tag}.samples")) == 0
        assert run("run", "import-emx", "--input", str(tmp_path / "g.txt"), "--output", str(tmp_path / f"{tag}.l.emx"),
                   "--nan", "NA", "--transform", "logarithm base 2") == 0
    assert (tmp_path / "py.emx").read_bytes() == (tmp_path / "native.emx").read_bytes()
    assert (tmp_path / "py.txt").read_text() == (tmp_path / "native.txt").read_text()
    assert (tmp_path / "py.l.emx").read_bytes() == (tmp_path / "native.l.emx").read_bytes()
    gem, genes, samples = pyoracle.import_emx_text(text, nan="NA")
    assert (tmp_path / "py.txt").read_text() == pyoracle.export_emx_text(gem, genes, samples, nan="NA")

    genes_n, maxk, S = _write_pair_files(tmp_path, rng)
    pm.export_text(tmp_path / "a.ccm", tmp_path / "a.cmx", tmp_path / "a.txt")
    for tag, run in runs.items():
        assert run("run", "import-cmx", "--input", str(tmp_path / "a.txt"), "--ccm", str(tmp_path / f"{tag}.ccm"),
                   "--cmx", str(tmp_path / f"{tag}.cmx"), "--genes", str(genes_n), "--maxclusters", str(maxk),
                   "--samples", str(S), "--corrname", "pearson") == 0
        assert (tmp_path / f"{tag}.ccm").read_bytes() == (tmp_path / "a.ccm").read_bytes()
    assert (tmp_path / "py.cmx").read_bytes() == (tmp_path / "native.cmx").read_bytes()
    # the reference requires a correlation name
    r = subprocess.run([exe, "run", "import-cmx", "--input", str(tmp_path / "a.txt"), "--ccm", "x", "--cmx", "y",
                        "--genes", "3", "--maxclusters", "2", "--samples", "7"], capture_output=True, text=True)
    assert r.returncode == 2


def test_reference_emx_text_tests(tmp_path, native):
    """KINC's own (disabled) import/export tests for expression matrices
    (tests/testimportexpressionmatrix.cpp, tests/testexportexpressionmatrix.cpp): a 10 x 5 matrix
    of values in [-10, 10), sample names on the first line, "NA" for missing values, text at the
    text stream's default 6 significant digits; the matrix read back within a mean error of 1e-3.
    Here the 6-digit text is also read bit-exactly as the restatement reads it, and the export
    (12 digits) reads back exactly."""
    rng = np.random.default_rng(11)
    gem = rng.uniform(-10, 10, (10, 5)).astype(np.float32)
    gem[2, 3] = np.nan
    lines = ["".join(f"{s}\t" for s in range(5))]
    lines += [str(g) + "".join("\tNA" if np.isnan(v) else "\t%.6g" % float(v) for v in gem[g]) for g in range(10)]
    text = "\n".join(lines) + "\n"
    (tmp_path / "t.txt").write_text(text)
    pm.import_emx_text(tmp_path / "t.txt", tmp_path / "t.emx", nan="NA")
    got = pm.read_emx(tmp_path / "t.emx")
    ok = ~np.isnan(gem)
    assert np.array_equal(np.isnan(got), ~ok) and np.abs(got[ok] - gem[ok]).mean() < 1e-3
    assert np.array_equal(got.view(np.uint32), pyoracle.import_emx_text(text, nan="NA")[0].view(np.uint32))
    pm.write_emx(tmp_path / "e.emx", gem)
    pm.export_emx_text(tmp_path / "e.emx", tmp_path / "e.txt", nan="NA")
    rows = [ln.split() for ln in (tmp_path / "e.txt").read_text().splitlines()]
    assert len(rows) == 11 and len(rows[0]) == 5 and all(len(r) == 6 for r in rows[1:])
    back = np.array([[np.nan if w == "NA" else float(w) for w in r[1:]] for r in rows[1:]], np.float32)
    assert np.array_equal(back.view(np.uint32), gem.view(np.uint32))
