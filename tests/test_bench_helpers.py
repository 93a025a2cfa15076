"""bench.py's host-side helpers: the parity block it reports and the clock-sample parsing
(fake nvidia-smi lines, no GPU)."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _results(n=6, S=5, seed=0):
    rng = np.random.default_rng(seed)
    K = rng.integers(0, 4, n).astype(np.int8)
    labels = rng.integers(-9, 3, (n, S)).astype(np.int8)
    corr = rng.uniform(-1, 1, (n, 5)).astype(np.float32)
    corr[np.arange(5)[None, :] >= K[:, None]] = np.nan
    return K, labels, corr


def test_parity_block_identical():
    r = _results()
    p = bench.parity_block(r, tuple(a.copy() for a in r))
    assert p["bit_exact"] and p["k_agreement"] == 1.0 and p["label_agreement"] == 1.0
    assert p["max_abs_dr"] == 0.0 and p["nan_mismatches"] == 0
    assert p["correlations"] == int(r[0].sum())
    assert sum(p["k_histogram"]) == len(r[0]) and p["k_histogram"][1] == int((r[0] == 1).sum())


def test_parity_block_reports_differences():
    K, L, C = _results(n=40, seed=3)
    K2, L2, C2 = K.copy(), L.copy(), C.copy()
    multi = np.nonzero(K > 1)[0]
    L2[multi[0], 0] ^= 1                              # one label string differs
    one = np.nonzero(K > 0)[0][0]
    C2[one, 0] += np.float32(1e-3)                    # one correlation differs
    p = bench.parity_block((K2, L2, C2), (K, L, C))
    assert not p["bit_exact"]
    assert abs(p["label_agreement"] - (1 - 1 / (K > 1).sum())) < 1e-12
    assert abs(p["max_abs_dr"] - 1e-3) < 1e-6
    K3 = K.copy()
    K3[0] = (K3[0] + 1) % 4                           # a K mismatch drops that pair from the comparisons
    p = bench.parity_block((K3, L, C), (K, L, C))
    assert abs(p["k_agreement"] - (1 - 1 / len(K))) < 1e-12 and not p["bit_exact"]


def test_clock_sampler_parses_smi_lines():
    s = bench.ClockSampler(0)
    s.proc = type("P", (), {"terminate": lambda self: None, "wait": lambda self, timeout=None: 0})()
    s.out = ["0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
             "0, 1980, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active",
             "0, 2070, 2070, 1000.0, 0x0, Not Active, Not Active, Not Active, Not Active",
             "garbage line"]
    c = s.stop()
    assert c["sm_mhz"] == 2070.0 and c["sm_max_mhz"] == 2070.0 and c["samples"] == 3
    assert c["reasons"] == ["sw_power_cap"]
