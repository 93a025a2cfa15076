"""The oracle (oracle/kinc_oracle.c) pinned against KINC's own code.

* glibc rand(): the restatement equals the C library's rand() stream.
* kinc_expf / kinc_logf: within 0.93 / 0.61 ulp of the true value.
* the restatement reproduces the golden fixtures (generated by KINC's own
  Pairwise:: sources, and by KINC's OpenCL kernels compiled for the host for
  the rand="lcg" mode, tests/golden/make_golden.py) bit for bit;
* when the KINC tree is present, it also equals KINC's compiled code on
  fresh cases, including blocks that start inside a work block.
"""
import glob
import json
import os

import numpy as np
import pytest

from kinc_gb300 import synthetic
from oracle import pyoracle

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def load_golden(path):
    """A fixture, plus corr_mask: the correlations the reference determines ([pair][cluster]; for the
    OpenCL worker's fixtures the clusters below K of the pairs in corr_rows, for the others every
    entry)."""
    z = np.load(path)
    g = dict(gem=z["gem"], K=z["K"], N=z["N"], corr=z["corr"], multi=z["multi"], labels=z["labels"],
             start=int(z["start"]), size=int(z["size"]), params=json.loads(str(z["params"])))
    if "corr_rows" in z.files:
        cols = np.arange(g["corr"].shape[1])[None, :]
        g["corr_mask"] = z["corr_rows"][:, None] & (cols < g["K"][:, None])
    else:
        g["corr_mask"] = np.ones(g["corr"].shape, bool)
    return g


def same_corr(a, b):
    return np.array_equal(np.nan_to_num(a, nan=9.0), np.nan_to_num(b, nan=9.0))


def test_rand_matches_libc():
    assert np.array_equal(pyoracle.rand_stream(50000), pyoracle.libc_rand(50000))


def test_rand_skip():
    full = pyoracle.libc_rand(5000)
    assert np.array_equal(pyoracle.rand_stream(100, skip=4321), full[4321:4421])


def test_fmath_accuracy():
    import ctypes
    L = ctypes.CDLL(pyoracle.build_ref.build_oracle())
    # exercise kinc_expf/kinc_logf through a tiny C harness compiled on the fly
    import subprocess
    import tempfile
    src = r'''
    #include "kinc_fmath.h"
    void f(const float* x, float* e, float* l, int n){ for(int i=0;i<n;++i){ e[i]=kinc_expf(x[i]); l[i]=kinc_logf(x[i]); } }
    '''
    d = tempfile.mkdtemp()
    with open(os.path.join(d, "h.c"), "w") as fh:
        fh.write(src)
    inc = os.path.join(os.path.dirname(os.path.dirname(__file__)), "kinc_gb300", "csrc")
    so = os.path.join(d, "h.so")
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-I", inc, "-o", so,
                           os.path.join(d, "h.c"), "-lm"])
    H = ctypes.CDLL(so)
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-104, 89, 200000), rng.uniform(-2, 2, 200000),
                        np.exp(rng.uniform(-100, 88, 200000)), rng.uniform(0.98, 1.03, 200000),
                        np.nextafter(np.float32(1), np.float32(0)) - np.arange(2000, dtype=np.float32) * 2 ** -24,
                        np.float32(1) + np.arange(2000, dtype=np.float32) * 2 ** -23]).astype(np.float32)
    e = np.empty_like(x)
    lg = np.empty_like(x)
    P = ctypes.c_void_p
    H.f(x.ctypes.data_as(P), e.ctypes.data_as(P), lg.ctypes.data_as(P), len(x))
    with np.errstate(over="ignore"):    # inputs past float's range are excluded below
        ex = np.exp(x.astype(np.float64))
        ulp = np.spacing(ex.astype(np.float32)).astype(np.float64)
    ok = (ex < 3.4e38) & (ex > 1.2e-38)
    assert np.max(np.abs(e[ok] - ex[ok]) / ulp[ok]) < 0.93
    pos = x > 0
    lx = np.log(x[pos].astype(np.float64))
    ulp = np.spacing(np.abs(lx).astype(np.float32)).astype(np.float64)
    nz = lx != 0
    assert np.max(np.abs(lg[pos][nz] - lx[nz]) / ulp[nz]) < 0.61
    specials = np.array([0.0, -0.0, 1.0, np.inf, -np.inf, np.nan, -1.0, 1e-45], np.float32)
    e = np.empty_like(specials)
    lg = np.empty_like(specials)
    H.f(specials.ctypes.data_as(P), e.ctypes.data_as(P), lg.ctypes.data_as(P), len(specials))
    assert e[0] == 1.0 and e[2] == np.float32(np.e) and e[3] == np.inf and e[4] == 0.0 and np.isnan(e[5])
    assert lg[0] == -np.inf and lg[2] == 0.0 and lg[3] == np.inf and np.isnan(lg[5]) and np.isnan(lg[6])
    assert abs(lg[7] - np.log(np.float64(specials[7]))) < 1e-4   # smallest subnormal


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_reproduces_golden(path):
    g = load_golden(path)
    p = pyoracle.params(**g["params"])
    K, labels, corr, N = pyoracle.run_block(g["gem"], p, g["start"], g["size"])
    assert np.array_equal(K, g["K"])
    assert np.array_equal(N, g["N"])
    assert np.array_equal(labels[g["multi"]], g["labels"])
    assert same_corr(corr[g["corr_mask"]], g["corr"][g["corr_mask"]])


REF_CASES = [
    (2, 260, 110, 32868, 300, dict(clus_method=1, corr_method=0, criterion=0, pre_out=1)),
    (5, 40, 70, 0, 780, dict(clus_method=1, corr_method=1, criterion=1, post_out=1, max_clusters=4)),
    (4, 36, 200, 0, 630, dict(clus_method=2, corr_method=1, criterion=0, max_clusters=3, pre_out=1, post_out=1)),
    (1, 270, 40, 30000, 6000, dict(min_expr=5.5)),
]


@pytest.mark.parametrize("case", REF_CASES)
def test_oracle_equals_compiled_reference(case):
    if pyoracle.ref_lib(0) is None:
        pytest.skip("KINC source tree not present: compiled reference unavailable")
    wl, G, S, start, size, kw = case
    gem = synthetic.generate(wl, genes=G, samples=S)
    size = min(size, G * (G - 1) // 2 - start)
    p = pyoracle.params(**kw)
    a = pyoracle.run_block(gem, p, start, size)
    b = pyoracle.run_ref(gem, p, (start // 32768) * 32768, start + size - (start // 32768) * 32768)
    off = start - (start // 32768) * 32768
    b = tuple(x[off:] for x in b)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[3], b[3])
    assert np.array_equal(a[1][a[0] > 1], b[1][b[0] > 1])
    assert same_corr(a[2], b[2])


def test_mid_block_start_replays_packed_array():
    gem = synthetic.generate(1, genes=60, samples=40)
    p = pyoracle.params()
    a = pyoracle.run_block(gem, p, 0, 1770)
    b = pyoracle.run_block(gem, p, 777, 993)
    assert same_corr(a[2][777:], b[2])


def test_process_matches_reference_rules():
    g = load_golden(GOLDEN[[os.path.basename(x) for x in GOLDEN].index("gmm_pearson_icl.npz")])
    p = pyoracle.params(**g["params"])
    K, labels, corr, _ = pyoracle.run_block(g["gem"], p, 0, g["size"])
    cmx, ccm = pyoracle.process_block(g["gem"].shape[1], p, 0, K, labels, corr)
    # every kept correlation passes the threshold and clusters are renumbered from 0 per pair
    assert np.all(np.abs(cmx["r"]) >= 0.5) and np.all(np.abs(cmx["r"]) <= 1.0)
    key = cmx["x"].astype(np.int64) * 100000 + cmx["y"]
    for k in np.unique(key):
        c = cmx["c"][key == k]
        assert np.array_equal(c, np.arange(len(c)))
    assert set(np.unique(ccm["codes"])) <= {0, 1, 6, 7, 8, 9}


def test_work_block_boundary_renews_packed_array():
    """Serial::execute runs once per 32768-pair work block with fresh arrays:
    a call spanning two blocks equals the two blocks run separately."""
    gem = synthetic.generate(1, genes=260, samples=36)
    p = pyoracle.params()
    both = pyoracle.run_block(gem, p, 32000, 1600)
    first = pyoracle.run_block(gem, p, 32000, 768)
    second = pyoracle.run_block(gem, p, 32768, 832)
    assert same_corr(both[2][:768], first[2]) and same_corr(both[2][768:], second[2])


def _edge_cases():
    import importlib.util
    import os
    path = os.path.join(os.path.dirname(__file__), "test_gpu_edge_cases.py")
    spec = importlib.util.spec_from_file_location("edge_cases_for_oracle", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.CASES


@pytest.mark.parametrize("case", _edge_cases(), ids=[c[0] for c in _edge_cases()])
def test_oracle_equals_compiled_reference_on_edge_inputs(case):
    """The restatement against KINC's own compiled Pairwise code on the GPU edge-case inputs
    (fits beyond five clusters, long sorts, degenerate genes, tiny matrices): the oracle the GPU
    edge tests compare with is itself pinned there."""
    if pyoracle.ref_lib(0) is None:
        pytest.skip("KINC source tree not present: compiled reference unavailable")
    name, make, _, oargs = case
    gem = make()
    G = gem.shape[0]
    total = G * (G - 1) // 2
    p = pyoracle.params(**oargs)
    a = pyoracle.run_block(gem, p, 0, total)
    b = pyoracle.run_ref(gem, p, 0, total)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[3], b[3])
    assert np.array_equal(a[1][a[0] > 1], b[1][b[0] > 1])
    assert same_corr(a[2], b[2])


def test_oracle_both_correlations_equal_two_runs():
    """corr_method 2 (Pearson and Spearman from one clustering, what the worker's corrmethod both
    computes) equals the two single-method runs a KINC user would make."""
    from kinc_gb300 import synthetic
    gem = synthetic.generate(5, genes=30, samples=90)
    kw = dict(clus_method=1, criterion=1, pre_out=1, post_out=1)
    Kb, Lb, Cb, Nb = pyoracle.run_block(gem, pyoracle.params(corr_method=2, **kw), 0, 300)
    for c in (0, 1):
        K, L, C, N = pyoracle.run_block(gem, pyoracle.params(corr_method=c, **kw), 0, 300)
        assert np.array_equal(K, Kb) and np.array_equal(L, Lb) and np.array_equal(N, Nb)
        assert np.array_equal(np.nan_to_num(C, nan=9.0), np.nan_to_num(Cb[:, :, c], nan=9.0))
