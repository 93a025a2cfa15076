"""RMT host side (include/kinc_rmt.h): the chi-square of the unfolded eigenvalue
spacings (computeChiSquare, src/core/rmt.cpp:289-439) against the oracle's
restatement, which unfolds with scipy's Akima spline.  Host code only."""
import numpy as np
import pytest

from kinc_gb300 import _native
from kinc_gb300.rmt import RMT
from oracle import pyoracle


def _spectrum(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "wishart":
        a = rng.standard_normal((n, 2 * n))
        w = np.linalg.eigvalsh(a @ a.T / (2 * n) + np.eye(n))
    else:   # uncorrelated levels
        w = np.sort(rng.uniform(0.5, 50.0, n))
    w = w[np.argsort(np.abs(w), kind="stable")]
    return w.astype(np.float32)


@pytest.mark.parametrize("kind", ["wishart", "poisson"])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_chi_square_matches_restatement(native, kind, seed):
    e = _spectrum(kind, 400, seed)
    rmt = RMT()
    got = rmt.chi_square(e)
    want = float(pyoracle.rmt_chi_square(e, pyoracle.RMT_DEFAULTS))
    assert got > 0
    assert abs(got - want) <= 1e-5 * abs(want), (got, want)


def test_chi_square_too_few_unique_values(native):
    e = np.repeat(np.float32([1.0, 2.0, 3.0]), 40)      # 120 values, 3 unique
    assert RMT().chi_square(e) == -1.0
    assert RMT().chi_square(np.arange(1, 50, dtype=np.float32)) == -1.0   # 48 unique after skipping the first


def test_chi_square_rejects_unordered_spectrum(native):
    e = np.linspace(-5, 5, 301).astype(np.float32)
    e = e[np.argsort(np.abs(e), kind="stable")]         # |lambda| order with both signs: not increasing
    with pytest.raises(_native.SimError) as err:
        RMT().chi_square(e)
    assert err.value.code == _native.RMT_ESPLINE


@pytest.mark.parametrize("kw", [dict(tstart=0.5, tstop=0.6), dict(minpace=40, maxpace=10)])
def test_invalid_arguments(native, kw):
    with pytest.raises(_native.SimError):
        RMT(**kw).chi_square(np.arange(100, dtype=np.float32))
