"""The command line (python -m kinc_gb300 run <analytic>) with KINC's analytic and
argument names: defaults, boolean arguments, and the host-only analytics end to end."""
import math

import numpy as np
import pytest

from kinc_gb300 import __main__ as cli, pairwise_matrix as pm


def _args(*argv):
    return cli._parser().parse_args(list(argv))


def test_similarity_defaults_are_the_references():
    a = _args("run", "similarity", "--input", "x.emx", "--cmx", "y.cmx")
    assert (a.clusmethod, a.corrmethod, a.minexpr, a.minsamp, a.minclus, a.maxclus, a.crit) == \
        ("none", "pearson", -math.inf, 30, 1, 5, "ICL")
    assert (a.preout, a.postout, a.mincorr, a.maxcorr, a.ksize) == (False, False, 0.5, 1.0, 4096)


@pytest.mark.parametrize("argv,want", [(["--preout"], True), (["--preout", "true"], True),
                                       (["--preout", "FALSE"], False), ([], False)])
def test_boolean_arguments(argv, want):
    assert _args("run", "similarity", "--input", "x", "--cmx", "y", *argv).preout is want


def test_resume_argument():
    assert _args("run", "similarity", "--input", "x", "--cmx", "y").resume is False
    assert _args("run", "similarity", "--input", "x", "--cmx", "y", "--resume").resume is True


def test_rand_mode_argument():
    assert _args("run", "similarity", "--input", "x", "--cmx", "y").rand == "glibc"
    assert _args("run", "similarity", "--input", "x", "--cmx", "y", "--rand", "lcg").rand == "lcg"
    with pytest.raises(SystemExit):
        _args("run", "similarity", "--input", "x", "--cmx", "y", "--rand", "mt")


def test_other_analytics_defaults():
    e = _args("run", "extract", "--emx", "a", "--ccm", "b", "--cmx", "c", "--output", "d")
    assert (e.mincorr, e.maxcorr) == (0.85, 1.0)
    r = _args("run", "rmt", "--input", "a", "--log", "b")
    assert (r.tstart, r.tstep, r.tstop, r.minpace, r.maxpace, r.bins) == (0.99, 0.001, 0.5, 10, 40, 60)


def test_export_and_extract_through_the_command_line(tmp_path, native):
    rng = np.random.default_rng(4)
    genes, samples = 9, 6
    gem = (8 + rng.standard_normal((genes, samples))).astype(np.float32)
    gem[0, 2] = np.nan
    pm.write_emx(tmp_path / "g.emx", gem)
    x, y, c = [3, 5, 5, 8], [1, 2, 2, 7], [0, 0, 1, 0]
    pm.write(tmp_path / "g.cmx", pm.CMX, genes, 3, 1, x, y, c, np.array([[0.9], [-0.95], [0.7], [0.99]], np.float32))
    pm.write(tmp_path / "g.ccm", pm.CCM, genes, 3, samples, [5, 5], [2, 2], [0, 1],
             np.array([[1, 1, 0, 9, 7, 8], [0, 0, 1, 6, 1, 1]], np.int8))
    assert cli.main(["run", "export-cmx", "--ccm", str(tmp_path / "g.ccm"), "--cmx", str(tmp_path / "g.cmx"),
                     "--output", str(tmp_path / "a.txt")]) == 0
    pm.export_text(tmp_path / "g.ccm", tmp_path / "g.cmx", tmp_path / "b.txt")
    assert (tmp_path / "a.txt").read_text() == (tmp_path / "b.txt").read_text()
    assert cli.main(["run", "extract", "--emx", str(tmp_path / "g.emx"), "--ccm", str(tmp_path / "g.ccm"),
                     "--cmx", str(tmp_path / "g.cmx"), "--output", str(tmp_path / "n.txt"),
                     "--graphml", str(tmp_path / "n.graphml")]) == 0
    lines = (tmp_path / "n.txt").read_text().splitlines()
    assert lines[0].startswith("Source\tTarget\tsc")
    assert [ln.split("\t")[:2] for ln in lines[1:]] == [["3", "1"], ["5", "2"], ["8", "7"]]   # |r| >= 0.85
    assert (tmp_path / "n.graphml").read_text().count("<edge ") == 3


def test_errors_are_reported_not_raised(tmp_path, native, capsys):
    assert cli.main(["run", "export-cmx", "--ccm", str(tmp_path / "none.ccm"), "--cmx", str(tmp_path / "none.cmx"),
                     "--output", str(tmp_path / "o.txt")]) == 1
    assert "export-cmx" in capsys.readouterr().err


def _native_cli():
    import os

    from kinc_gb300 import build
    if not os.path.exists(build.CLI):
        pytest.skip("command-line program not built")
    return build.CLI


def test_native_program_export_and_extract(tmp_path, native):
    """kinc-gb300 (the C++ host driver) writes what the library calls write."""
    import subprocess
    exe = _native_cli()
    rng = np.random.default_rng(8)
    genes, samples = 7, 5
    gem = (8 + rng.standard_normal((genes, samples))).astype(np.float32)
    pm.write_emx(tmp_path / "g.emx", gem)
    pm.write(tmp_path / "g.cmx", pm.CMX, genes, 2, 1, [2, 4, 4], [1, 3, 3], [0, 0, 1],
             np.array([[0.9], [0.95], [-0.88]], np.float32))
    pm.write(tmp_path / "g.ccm", pm.CCM, genes, 2, samples, [4, 4], [3, 3], [0, 1],
             np.array([[1, 1, 0, 9, 7], [0, 0, 1, 6, 1]], np.int8))
    r = subprocess.run([exe, "run", "export-cmx", "--ccm", str(tmp_path / "g.ccm"), "--cmx", str(tmp_path / "g.cmx"),
                        "--output", str(tmp_path / "a.txt")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pm.export_text(tmp_path / "g.ccm", tmp_path / "g.cmx", tmp_path / "b.txt")
    assert (tmp_path / "a.txt").read_text() == (tmp_path / "b.txt").read_text()
    r = subprocess.run([exe, "run", "extract", "--emx", str(tmp_path / "g.emx"), "--ccm", str(tmp_path / "g.ccm"),
                        "--cmx", str(tmp_path / "g.cmx"), "--output", str(tmp_path / "n1.txt"),
                        "--mincorr", "0.85"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pm.extract(tmp_path / "g.emx", tmp_path / "g.ccm", tmp_path / "g.cmx", tsv_path=tmp_path / "n2.txt")
    assert (tmp_path / "n1.txt").read_text() == (tmp_path / "n2.txt").read_text()


@pytest.mark.parametrize("argv,code", [([], 2), (["run"], 2), (["run", "nope"], 2),
                                       (["run", "similarity", "--input"], 2),
                                       (["run", "similarity", "--input", "x.emx"], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--preout", "maybe"], 2),
                                       (["run", "export-cmx", "--ccm", "a", "--cmx", "b", "--output", "c"], 1),
                                       # unknown and malformed arguments are usage errors, as in argparse
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--minsmap", "3"], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--minsamp", "3x"], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--blocks", ""], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--rand", "mt"], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--world", "2",
                                         "--rank", "2"], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--world", "2",
                                         "--first-block", "1"], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--by-cost"], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--resume",
                                         "maybe"], 2),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--resume"], 1),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--world", "2",
                                         "--rank", "1", "--by-cost"], 1),
                                       (["run", "similarity", "--input", "x.emx", "--cmx", "y", "--rand", "lcg"], 1),
                                       (["run", "extract", "--emx", "a", "--ccm", "b", "--cmx", "c", "--output", "d",
                                         "--mincorr", "high"], 2),
                                       (["run", "rmt", "--input", "a", "--log", "b", "--bins", "1e9"], 2),
                                       (["run", "rmt", "--input", "a", "--log", "b", "--bins", "99999999999"], 2),
                                       (["run", "export-cmx", "--ccm", "a", "--cmx", "b", "--output", "c",
                                         "--preout"], 2),
                                       (["run", "import-cmx", "--input", "a", "--ccm", "b", "--cmx", "c", "--genes",
                                         "5", "--maxclusters", "2", "--samples", "4"], 2),
                                       (["run", "import-emx", "--input", "a", "--output", "b", "--transform", "log"],
                                        2)])
def test_native_program_argument_errors(tmp_path, native, argv, code):
    import subprocess
    r = subprocess.run([_native_cli(), *argv], capture_output=True, text=True, cwd=tmp_path)
    assert r.returncode == code, r.stderr


@pytest.mark.parametrize("argv", [["run", "similarity", "--input", "x", "--cmx", "y", "--minsmap", "3"],
                                  ["run", "similarity", "--input", "x", "--cmx", "y", "--minsamp", "3x"],
                                  ["run", "import-emx", "--input", "a", "--output", "b", "--transform", "log"]])
def test_python_command_line_rejects_what_the_native_one_rejects(argv):
    with pytest.raises(SystemExit) as e:
        cli._parser().parse_args(argv)
    assert e.value.code == 2


def test_merge_through_both_command_lines(tmp_path, native):
    import subprocess
    x, y, c = [2, 3, 3, 5], [1, 0, 0, 4], [0, 0, 1, 0]
    r = np.array([[0.9], [-0.8], [0.7], [0.6]], np.float32)
    pm.write(tmp_path / "all.cmx", pm.CMX, 6, 2, 1, x, y, c, r)
    pm.write(tmp_path / "r0.cmx", pm.CMX, 6, 2, 1, x[:2], y[:2], c[:2], r[:2])
    pm.write(tmp_path / "r1.cmx", pm.CMX, 6, 2, 1, x[2:], y[2:], c[2:], r[2:])
    ins = [str(tmp_path / "r0.cmx"), str(tmp_path / "r1.cmx")]
    assert cli.main(["run", "merge", "--output", str(tmp_path / "py.cmx"), "--inputs", *ins]) == 0
    res = subprocess.run([_native_cli(), "run", "merge", "--output", str(tmp_path / "nat.cmx"), "--inputs",
                          ",".join(ins)], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    want = (tmp_path / "all.cmx").read_bytes()
    assert (tmp_path / "py.cmx").read_bytes() == want and (tmp_path / "nat.cmx").read_bytes() == want
