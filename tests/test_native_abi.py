"""The C ABI library: it loads, exports every function include/*.h
declares, validates arguments, and its host-only filter (Similarity::process)
matches the oracle.  No kernel is launched here."""
import ctypes
import os
import re

import numpy as np
import pytest

from kinc_gb300 import _native, synthetic
from oracle import pyoracle

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for f in sorted(os.listdir(INCLUDE)):
        if f.endswith(".h"):
            text = re.sub(r"/\*.*?\*/", "", open(os.path.join(INCLUDE, f)).read(), flags=re.S)
            names |= set(re.findall(r"\b(kinc_\w+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(native):
    names = declared_symbols()
    assert len(names) >= 25
    for n in names:
        assert hasattr(native, n), n
        assert n in _native.SIGNATURES, n


def test_params_default_matches_reference_defaults(native):
    p = _native.SimParams()
    assert native.kinc_sim_params_default(ctypes.byref(p)) == 0
    assert (p.clus_method, p.corr_method, p.min_samples, p.min_clusters, p.max_clusters, p.criterion) == \
        (0, 0, 30, 1, 5, 1)
    assert p.min_expr == float("-inf") and p.pre_out == 0 and p.post_out == 0 and p.ksize == 4096
    assert abs(p.min_corr - 0.5) < 1e-7 and p.max_corr == 1.0


@pytest.mark.parametrize("field,value", [("min_clusters", 3), ("min_samples", 0), ("clus_method", 7),
                                         ("max_clusters", 65), ("min_corr", 1.5), ("precision", 5)])
def test_create_rejects_invalid_arguments(native, field, value):
    p = _native.SimParams()
    native.kinc_sim_params_default(ctypes.byref(p))
    if field == "min_clusters":
        p.max_clusters = 2
    setattr(p, field, value)
    gem = np.zeros((4, 8), np.float32)
    ctx = ctypes.c_void_p()
    rc = native.kinc_sim_create(gem.ctypes.data_as(ctypes.c_void_p), 4, 8, ctypes.byref(p), ctypes.byref(ctx))
    assert rc == _native.EINVAL
    assert native.kinc_sim_last_error(None)
    if field == "min_clusters":
        assert b"Minimum clusters must be less than or equal to maximum clusters." in \
            native.kinc_sim_last_error(None)


@pytest.mark.parametrize("precision", [1, 2, 3, 4])
def test_contraction_precisions_need_pairwise_complete_pearson(native, precision):
    """The tensor-core and tiled precisions compute the pairwise-complete Pearson contraction only:
    clus_method none, corr_method pearson, semantics 1 (each sample's own values)."""
    p = _native.SimParams()
    native.kinc_sim_params_default(ctypes.byref(p))
    p.precision = precision
    p.clus_method = 1
    gem = np.zeros((4, 8), np.float32)
    ctx = ctypes.c_void_p()
    rc = native.kinc_sim_create(gem.ctypes.data_as(ctypes.c_void_p), 4, 8, ctypes.byref(p), ctypes.byref(ctx))
    assert rc == _native.EINVAL
    assert b"pairwise-complete Pearson contraction" in native.kinc_sim_last_error(None)


def _process_native(native, p, S, start, K, labels, corr):
    size = len(K)
    cap = size * p.max_clusters
    cx, cy, cc, cr = (np.empty(cap, np.int32), np.empty(cap, np.int32), np.empty(cap, np.int8),
                      np.empty(cap, np.float32))
    mx, my, mc = np.empty(cap, np.int32), np.empty(cap, np.int32), np.empty(cap, np.int8)
    codes = np.empty((cap, S), np.int8)
    n1, n2 = ctypes.c_int64(), ctypes.c_int64()
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = native.kinc_sim_process_pairs(ctypes.byref(p), S, start, size, vp(K), vp(labels), vp(corr), vp(cx),
                                       vp(cy), vp(cc), vp(cr), cap, ctypes.byref(n1), vp(mx), vp(my), vp(mc),
                                       vp(codes), cap, ctypes.byref(n2))
    assert rc == 0
    return (dict(x=cx[:n1.value], y=cy[:n1.value], c=cc[:n1.value], r=cr[:n1.value]),
            dict(x=mx[:n2.value], y=my[:n2.value], c=mc[:n2.value], codes=codes[:n2.value]))


def test_process_pairs_matches_oracle(native):
    gem = synthetic.generate(2, genes=30, samples=80)
    op = pyoracle.params(clus_method=1, corr_method=0, criterion=1, min_corr=0.3)
    K, labels, corr, _ = pyoracle.run_block(gem, op, 0, 435)
    p = _native.SimParams()
    native.kinc_sim_params_default(ctypes.byref(p))
    p.clus_method, p.corr_method, p.criterion, p.min_corr = 1, 0, 1, 0.3
    got = _process_native(native, p, 80, 0, K, labels, corr)
    want = pyoracle.process_block(80, op, 0, K, labels, corr)
    for g, w in zip(got, want):
        for key in w:
            assert np.array_equal(g[key], w[key]), key


def test_process_pairs_capacity_error(native):
    p = _native.SimParams()
    native.kinc_sim_params_default(ctypes.byref(p))
    K = np.ones(4, np.int8)
    corr = np.full((4, 5), 0.9, np.float32)
    one = np.empty(1, np.int32)
    n = ctypes.c_int64()
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = native.kinc_sim_process_pairs(ctypes.byref(p), 8, 0, 4, vp(K), None, vp(corr), vp(one), vp(one),
                                       vp(np.empty(1, np.int8)), vp(np.empty(1, np.float32)), 1,
                                       ctypes.byref(n), None, None, None, None, 0, None)
    assert rc == _native.EINVAL
