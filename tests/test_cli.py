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
