"""The RMT analytic on the GPU (include/kinc_rmt.h) against the oracle's
restatement of RMT::process (numpy eigensolver, scipy Akima unfolding):
pruned-matrix eigenvalues, the (threshold, size, chi) sequence, the result or
the reference's failure, and the log file."""
import numpy as np
import pytest

from kinc_gb300 import _native, pairwise_matrix as pm, synthetic
from kinc_gb300.rmt import RMT
from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _random_network(G, K, seed, frac=0.05):
    rng = np.random.default_rng(seed)
    xs, ys, cs, rs = [], [], [], []
    for x in range(1, G):
        for y in range(x):
            for k in range(K):
                if rng.random() < frac:
                    xs.append(x); ys.append(y); cs.append(k); rs.append(rng.uniform(0.5, 1.0) * rng.choice([-1, 1]))
    return G, np.array(xs, np.int32), np.array(ys, np.int32), np.array(cs, np.int8), np.array(rs, np.float32)


@pytest.mark.parametrize("net,threshold", [("cliques", 0.9), ("cliques", 0.75), ("random", 0.8), ("random", 0.6)])
def test_pruned_eigenvalues_match_numpy(net, threshold):
    if net == "cliques":
        G, x, y, c, r = synthetic.clique_network(60, 6)
        K = 1
    else:
        K = 2
        G, x, y, c, r = _random_network(120, K, 5)
    got = RMT().prune_eigenvalues((x, y, c, r), G, K, threshold)
    mat = pyoracle.rmt_dense(G, K, x, y, c, r)
    want = pyoracle.rmt_prune_eigenvalues(mat, pyoracle.rmt_maximums(mat), threshold)
    assert len(got) == len(want) > 0
    assert np.allclose(got, want, rtol=0, atol=1e-5 * max(1.0, float(np.abs(want).max())))


@pytest.mark.parametrize("chi", [(99.607, 200.0), (50.0, 55.0)])
def test_run_matches_oracle(chi):
    """Default chi-square limits: no threshold above 0.6 (the reference's error); tighter ones: a result."""
    G, x, y, c, r = synthetic.clique_network(80, 5)
    args = dict(threshold_step=0.01, threshold_stop=0.6, chi_square_threshold1=chi[0], chi_square_threshold2=chi[1])
    want_t, want_steps = pyoracle.rmt_run(G, 1, x, y, c, r, **args)
    rmt = RMT(tstep=0.01, tstop=0.6, chi1=chi[0], chi2=chi[1])
    if want_t is None:
        with pytest.raises(_native.SimError) as err:
            rmt.run(items=(x, y, c, r), genes=G, max_clusters=1)
        assert err.value.code == _native.RMT_ENOTHRESHOLD
        return
    got_t, steps = rmt.run(items=(x, y, c, r), genes=G, max_clusters=1)
    assert len(steps) == len(want_steps)
    for (t1, m1, c1), (t2, m2, c2) in zip(steps, want_steps):
        assert np.float32(t1) == np.float32(t2) and int(m1) == m2
        assert abs(c1 - c2) <= 1e-4 * max(1.0, abs(c2)), (t1, c1, c2)
    assert np.float32(got_t) == np.float32(want_t)


def test_run_from_cmx_file_writes_the_log(tmp_path):
    G, x, y, c, r = synthetic.clique_network(80, 5)
    pm.write(tmp_path / "n.cmx", pm.CMX, G, 1, 1, x, y, c, r.reshape(-1, 1))
    rmt = RMT(tstep=0.01, tstop=0.6, chi1=50.0, chi2=55.0)
    t, _ = rmt.run(input=tmp_path / "n.cmx", log=tmp_path / "rmt.log")
    want_t, want_steps = pyoracle.rmt_run(G, 1, x, y, c, r, threshold_step=0.01, threshold_stop=0.6,
                                          chi_square_threshold1=50.0, chi_square_threshold2=55.0)
    lines = (tmp_path / "rmt.log").read_text().splitlines()
    assert len(lines) == len(want_steps) + 1
    for line, (ts, m, chi) in zip(lines, want_steps):
        a, b, cc = line.split("\t")
        assert a == "%.6g" % np.float32(ts) and int(b) == m
        assert abs(float(cc) - chi) <= 1e-3 * max(1.0, abs(chi))
    assert lines[-1] == "%.6g" % np.float32(want_t)
    assert np.float32(t) == np.float32(want_t)


def test_spline_failure_matches_oracle():
    """A network whose pruned matrices have negative eigenvalues: the unfolding's knots do not increase in
    |lambda| order, which the reference's spline library rejects; both sides stop at the same step."""
    G, x, y, c, r = _random_network(150, 1, 9, frac=0.2)
    with pytest.raises(pyoracle.RMTSplineError):
        pyoracle.rmt_run(G, 1, x, y, c, r, threshold_step=0.01)
    with pytest.raises(_native.SimError) as err:
        RMT(tstep=0.01).run(items=(x, y, c, r), genes=G, max_clusters=1)
    assert err.value.code == _native.RMT_ESPLINE
