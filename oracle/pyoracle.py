"""ctypes bindings for the CPU checkers (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this module.  It wraps:

* the C restatement (``libkinc_oracle.so``, built from kinc_oracle.c), and
* KINC's own Pairwise:: sources compiled by build_ref.py
  (``oracle/_ref/libkinc_ref{0,1,2}.so``), when the KINC tree was available
  to build them.
"""
import ctypes
import os

import numpy as np

from . import build_ref

HERE = os.path.dirname(os.path.abspath(__file__))


class KoParams(ctypes.Structure):
    _fields_ = [("clus_method", ctypes.c_int32), ("corr_method", ctypes.c_int32),
                ("min_expr", ctypes.c_float), ("min_samples", ctypes.c_int32),
                ("min_clusters", ctypes.c_int32), ("max_clusters", ctypes.c_int32),
                ("criterion", ctypes.c_int32), ("pre_out", ctypes.c_int32),
                ("post_out", ctypes.c_int32), ("min_corr", ctypes.c_float),
                ("max_corr", ctypes.c_float), ("semantics", ctypes.c_int32),
                ("rand_mode", ctypes.c_int32)]


class KoRand(ctypes.Structure):
    _fields_ = [("r", ctypes.c_uint32 * 34), ("head", ctypes.c_int32), ("drawn", ctypes.c_uint64)]


_lib = None
_ref = {}


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build_oracle()
        L = ctypes.CDLL(path)
        P = ctypes.POINTER
        L.ko_rand_seed.argtypes = [P(KoRand), ctypes.c_uint32]
        L.ko_rand_next.argtypes = [P(KoRand)]
        L.ko_rand_next.restype = ctypes.c_int32
        L.ko_rand_skip.argtypes = [P(KoRand), ctypes.c_uint64]
        L.ko_libc_rand.argtypes = [ctypes.c_uint32, ctypes.c_int32, P(ctypes.c_int32)]
        L.ko_draws_per_pair.argtypes = [P(KoParams)]
        L.ko_draws_per_pair.restype = ctypes.c_int64
        L.ko_count_qualifying.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, P(KoParams),
                                          ctypes.c_int64]
        L.ko_count_qualifying.restype = ctypes.c_int64
        L.ko_run_block.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, P(KoParams), P(KoRand),
                                   ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p]
        L.ko_run_block.restype = ctypes.c_int
        L.ko_run_segments_parallel.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, P(KoParams),
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_int32, ctypes.c_int32, P(ctypes.c_double)]
        L.ko_run_segments_parallel.restype = ctypes.c_int64
        L.ko_run_segments_parallel_out.argtypes = L.ko_run_segments_parallel.argtypes + [ctypes.c_void_p] * 3
        L.ko_run_segments_parallel_out.restype = ctypes.c_int64
        L.ko_process_block.argtypes = [ctypes.c_int32, P(KoParams), ctypes.c_int64, ctypes.c_int64,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p] + \
            [ctypes.c_void_p] * 8 + [P(ctypes.c_int64)]
        L.ko_process_block.restype = ctypes.c_int64
        L.ko_pearson_fp64.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                      ctypes.c_float, ctypes.c_int32]
        L.ko_pearson_fp64.restype = ctypes.c_double
        L.ko_pearson_fp64_batch.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int64, ctypes.c_float, ctypes.c_int32, ctypes.c_void_p,
                                            ctypes.c_int32]
        _lib = L
    return _lib


def ref_lib(math_mode=0):
    """KINC's compiled Pairwise:: sources, or None if the KINC tree is absent."""
    if math_mode not in _ref:
        path = build_ref.build_ref(math_mode)
        if path is None:
            _ref[math_mode] = None
        else:
            L = ctypes.CDLL(path)
            L.kinc_ref_run_block.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + \
                [ctypes.c_int, ctypes.c_int, ctypes.c_float] + [ctypes.c_int] * 6 + \
                [ctypes.c_int64, ctypes.c_int64, ctypes.c_uint64] + [ctypes.c_void_p] * 4
            L.kinc_ref_run_block.restype = ctypes.c_int
            _ref[math_mode] = L
    return _ref[math_mode]


DEFAULTS = dict(clus_method=0, corr_method=0, min_expr=float("-inf"), min_samples=30, min_clusters=1,
                max_clusters=5, criterion=1, pre_out=0, post_out=0, min_corr=0.5, max_corr=1.0,
                semantics=0, rand_mode=0)


def params(**kw):
    d = dict(DEFAULTS)
    d.update(kw)
    p = KoParams()
    for k, v in d.items():
        setattr(p, k, v)
    return p


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def rand_position(gem, p, start):
    """Draws a fresh serial KINC process has taken from rand() before pair `start`."""
    L = lib()
    G, S = gem.shape
    per = L.ko_draws_per_pair(ctypes.byref(p))
    if per == 0 or start == 0:
        return 0
    return per * L.ko_count_qualifying(_ptr(gem), G, S, ctypes.byref(p), start)


def run_block(gem, p, start, size, rand_pos=None):
    """The C restatement of Similarity::Serial::execute over [start, start+size)."""
    L = lib()
    gem = np.ascontiguousarray(gem, dtype=np.float32)
    G, S = gem.shape
    K = np.zeros(size, np.int8)
    labels = np.zeros((size, S), np.int8)
    corr = np.zeros((size, p.max_clusters), np.float32)
    N = np.zeros(size, np.int32)
    g = KoRand()
    L.ko_rand_seed(ctypes.byref(g), 1)
    pos = rand_position(gem, p, start) if rand_pos is None else rand_pos
    L.ko_rand_skip(ctypes.byref(g), pos)
    rc = L.ko_run_block(_ptr(gem), G, S, ctypes.byref(p), ctypes.byref(g), start, size, _ptr(K), _ptr(labels),
                        _ptr(corr), _ptr(N))
    if rc != 0:
        raise ValueError("oracle rejected the arguments")
    return K, labels, corr, N


def run_ref(gem, p, start, size, math_mode=0, rand_pos=None):
    """KINC's own models over [start, start+size), or None when not built."""
    R = ref_lib(math_mode)
    if R is None:
        return None
    gem = np.ascontiguousarray(gem, dtype=np.float32)
    G, S = gem.shape
    K = np.zeros(size, np.int8)
    labels = np.zeros((size, S), np.int8)
    corr = np.zeros((size, p.max_clusters), np.float32)
    N = np.zeros(size, np.int32)
    pos = rand_position(gem, p, start) if rand_pos is None else rand_pos
    R.kinc_ref_run_block(_ptr(gem), G, S, p.clus_method, p.corr_method, p.min_expr, p.min_samples,
                         p.min_clusters, p.max_clusters, p.criterion, p.pre_out, p.post_out, start, size, pos,
                         _ptr(K), _ptr(labels), _ptr(corr), _ptr(N))
    return K, labels, corr, N


def process_block(S, p, start, K, labels, corr):
    """Similarity::process restated: (cmx items, ccm items) as dicts of arrays."""
    L = lib()
    size = len(K)
    cap = size * p.max_clusters
    cx, cy, cc, cr = (np.zeros(cap, np.int32), np.zeros(cap, np.int32), np.zeros(cap, np.int8),
                      np.zeros(cap, np.float32))
    mx, my, mc, codes = (np.zeros(cap, np.int32), np.zeros(cap, np.int32), np.zeros(cap, np.int8),
                         np.zeros((cap, S), np.int8))
    n_ccm = ctypes.c_int64(0)
    n_cmx = L.ko_process_block(S, ctypes.byref(p), start, size, _ptr(np.ascontiguousarray(K)),
                               _ptr(np.ascontiguousarray(labels)), _ptr(np.ascontiguousarray(corr)),
                               _ptr(cx), _ptr(cy), _ptr(cc), _ptr(cr), _ptr(mx), _ptr(my), _ptr(mc), _ptr(codes),
                               ctypes.byref(n_ccm))
    m = n_ccm.value
    return (dict(x=cx[:n_cmx], y=cy[:n_cmx], c=cc[:n_cmx], r=cr[:n_cmx]),
            dict(x=mx[:m], y=my[:m], c=mc[:m], codes=codes[:m]))


def run_segments_parallel(gem, p, starts, sizes, threads, outputs=False):
    """Time the restatement over segments with POSIX threads; returns (pairs, seconds), plus
    (K, labels, corr) of the segments back to back when `outputs` is set."""
    L = lib()
    gem = np.ascontiguousarray(gem, dtype=np.float32)
    G, S = gem.shape
    starts = np.ascontiguousarray(starts, dtype=np.int64)
    sizes = np.ascontiguousarray(sizes, dtype=np.int64)
    pos = np.array([rand_position(gem, p, int(s)) for s in starts], dtype=np.uint64)
    secs = ctypes.c_double(0)
    if not outputs:
        done = L.ko_run_segments_parallel(_ptr(gem), G, S, ctypes.byref(p), _ptr(starts), _ptr(sizes), _ptr(pos),
                                          len(starts), threads, ctypes.byref(secs))
        return done, secs.value
    n = int(sizes.sum())
    K = np.zeros(n, np.int8)
    labels = np.zeros((n, S), np.int8)
    corr = np.zeros((n, p.max_clusters), np.float32)
    done = L.ko_run_segments_parallel_out(_ptr(gem), G, S, ctypes.byref(p), _ptr(starts), _ptr(sizes), _ptr(pos),
                                          len(starts), threads, ctypes.byref(secs), _ptr(K), _ptr(labels),
                                          _ptr(corr))
    return done, secs.value, (K, labels, corr)


def pearson_fp64(gem, x, y, min_expr=float("-inf"), min_samples=30):
    gem = np.ascontiguousarray(gem, dtype=np.float32)
    return lib().ko_pearson_fp64(_ptr(gem), gem.shape[1], x, y, min_expr, min_samples)


def pearson_fp64_pairs(gem, xs, ys, min_expr=float("-inf"), min_samples=30):
    """FP64 pairwise-complete Pearson for the pairs (xs[i], ys[i])."""
    gem = np.ascontiguousarray(gem, dtype=np.float32)
    xs = np.ascontiguousarray(xs, dtype=np.int32)
    ys = np.ascontiguousarray(ys, dtype=np.int32)
    out = np.empty(len(xs), np.float64)
    lib().ko_pearson_fp64_batch(_ptr(gem), gem.shape[1], _ptr(xs), _ptr(ys), len(xs), min_expr, min_samples,
                                _ptr(out), os.cpu_count() or 1)
    return out


def pair_xy(p):
    """Vectorised linear pair index -> (x, y), x > y."""
    p = np.asarray(p, dtype=np.int64)
    x = ((1 + np.sqrt(1 + 8 * p.astype(np.float64))) // 2).astype(np.int64)
    x -= (x * (x - 1) // 2 > p)
    x += ((x + 1) * x // 2 <= p)
    return x, p - x * (x - 1) // 2


def libc_rand(n, seed=1):
    out = (ctypes.c_int32 * n)()
    lib().ko_libc_rand(seed, n, out)
    return np.frombuffer(out, dtype=np.int32).copy()


def rand_stream(n, seed=1, skip=0):
    L = lib()
    g = KoRand()
    L.ko_rand_seed(ctypes.byref(g), seed)
    L.ko_rand_skip(ctypes.byref(g), skip)
    return np.array([L.ko_rand_next(ctypes.byref(g)) for _ in range(n)], dtype=np.int32)


def export_text(cmx, ccm, S):
    """ExportCorrelationMatrix::process restated (src/core/exportcorrelationmatrix.cpp:17-117) over
    item dicts as pairwise_matrix.read returns them; returns the text."""
    lines = []
    n = len(cmx["x"])
    ccm_at = {}
    for q in range(len(ccm["x"])):
        ccm_at.setdefault((int(ccm["x"][q]), int(ccm["y"][q])), []).append(ccm["payload"][q])
    i = 0
    while i < n:
        x, y = int(cmx["x"][i]), int(cmx["y"][i])
        j = i
        while j < n and int(cmx["x"][j]) == x and int(cmx["y"][j]) == y:
            j += 1
        size = j - i
        for k in range(size):
            r = float(cmx["payload"][i + k][0])
            counts = {1: 0, 6: 0, 7: 0, 8: 0, 9: 0}
            if size > 1:
                codes = ccm_at[(x, y)][k]
                for c in codes:
                    if int(c) in counts:
                        counts[int(c)] += 1
                mask = "".join(chr(ord("0") + int(c)) for c in codes)
            else:
                mask = "0" * S
            lines.append(f"{x}\t{y}\t{k}\t{size}\t{counts[1]}\t{counts[9]}\t{counts[8]}\t{counts[7]}\t"
                         f"{counts[6]}\t{'%.6g' % r}\t{mask}\n")
        i = j
    return "".join(lines)


def extract_network(gem, cmx, ccm, S, names=None, min_corr=0.85, max_corr=1.0):
    """Extract::process restated (src/core/extract.cpp:24-274) over item dicts as
    pairwise_matrix.read returns them; returns (tsv text, graphml text)."""
    G = gem.shape[0]
    names = [str(g) for g in range(G)] if names is None else list(names)
    lo, hi = np.float32(min_corr), np.float32(max_corr)
    tsv = ["Source\tTarget\tsc\tInteraction\tCluster\tNum_Clusters\tCluster_Samples\tMissing_Samples\t"
           "Cluster_Outliers\tPair_Outliers\tToo_Low\tSamples\n"]
    gml = ['<?xml version="1.0" encoding="UTF-8"?>\n',
           '<graphml xmlns="http://graphml.graphdrawing.org/xmlns"\n',
           '    xmlns:xsi="http://www.w3.org/2001/XMLSchema-instance"\n',
           '    xsi:schemaLocation="http://graphml.graphdrawing.org/xmlns/1.0/graphml.xsd">\n',
           '  <graph id="G" edgedefault="undirected">\n']
    gml += [f'    <node id="{names[g]}"/>\n' for g in range(G)]
    ccm_at = {}
    for q in range(len(ccm["x"])):
        ccm_at.setdefault((int(ccm["x"][q]), int(ccm["y"][q])), []).append(ccm["payload"][q])
    n = len(cmx["x"])
    i = 0
    while i < n:
        x, y = int(cmx["x"][i]), int(cmx["y"][i])
        j = i
        while j < n and int(cmx["x"][j]) == x and int(cmx["y"][j]) == y:
            j += 1
        size = j - i
        for k in range(size):
            r = np.float32(cmx["payload"][i + k][0])
            if abs(r) < lo or hi < abs(r):
                continue
            counts = {1: 0, 6: 0, 7: 0, 8: 0, 9: 0}
            if size > 1:
                codes = ccm_at[(x, y)][k]
                for c in codes:
                    if int(c) in counts:
                        counts[int(c)] += 1
                mask = "".join(chr(ord("0") + int(c)) for c in codes)
            else:
                mask = "".join("9" if (np.isnan(gem[x, s]) or np.isnan(gem[y, s])) else "1" for s in range(S))
            tsv.append(f"{names[x]}\t{names[y]}\t{'%.6g' % float(r)}\tco\t{k}\t{size}\t{counts[1]}\t{counts[9]}\t"
                       f"{counts[8]}\t{counts[7]}\t{counts[6]}\t{mask}\n")
            gml.append(f'    <edge source="{names[x]}" target="{names[y]}" samples="{mask}"/>\n')
        i = j
    gml.append("  </graph>\n</graphml>\n")
    return "".join(tsv), "".join(gml)


# ----------------------------------------------------------------------------- RMT
# RMT::process and its helpers restated (src/core/rmt.cpp:33-122,164-439) with numpy:
# the dense pruned matrix, LAPACK's symmetric eigensolver (numpy.linalg.eigvalsh on
# the lower triangle, double), scipy's Akima spline for the unfolding, float32 where
# the reference keeps floats.

RMT_DEFAULTS = dict(threshold_start=0.99, threshold_step=0.001, threshold_stop=0.5, chi_square_threshold1=99.607,
                    chi_square_threshold2=200.0, min_eigenvalue_size=50, min_unfolding_pace=10,
                    max_unfolding_pace=40, histogram_bin_size=60)


class RMTSplineError(ValueError):
    """The unfolding spline got knots that do not increase (the reference's spline library rejects them)."""


def rmt_dense(G, K, x, y, c, r):
    """CorrelationMatrix::dumpRawData (src/core/correlationmatrix.cpp:144-177): [G][G][K], zeros elsewhere."""
    m = np.zeros((G, G, K), np.float32)
    m[x, y, c] = r
    m[y, x, c] = r
    return m


def rmt_maximums(mat):
    """computeMaximums: per (gene, cluster) the largest |r| over the other genes (0 when none)."""
    a = np.abs(mat)
    a = np.where(np.isnan(a), 0, a)
    return a.max(axis=1).reshape(-1)


def rmt_prune_eigenvalues(mat, maximums, threshold):
    """computePruneMatrix + computeEigenvalues: eigenvalues sorted by ascending |lambda|, as float32."""
    G, _, K = mat.shape
    t = np.float32(threshold)
    idx = np.nonzero(maximums >= t)[0]
    m = len(idx)
    if m == 0:
        return np.zeros(0, np.float32)
    P = np.zeros((m, m), np.float64)
    gi, ki = idx // K, idx % K
    for i in range(m):
        js = np.arange(i)
        same = ki[js] == ki[i]
        js = js[same]
        v = mat[gi[i], gi[js], ki[i]]
        keep = np.abs(v) >= t
        P[i, js[keep]] = v[keep]
        P[i, i] = 1.0
    w = np.linalg.eigvalsh(P, UPLO="L")
    order = np.argsort(np.abs(w), kind="stable")
    return w[order].astype(np.float32)


def rmt_chi_square(eigens, p):
    """computeChiSquare / computePaceChiSquare / degenerate / unfold; -1 with too few unique values."""
    from scipy.interpolate import Akima1DInterpolator
    e = [np.float32(v) for v in eigens]
    uniq = []
    for i in range(1, len(e)):
        if not uniq or abs(np.float32(e[i] - uniq[-1])) > np.float32(1e-6):
            uniq.append(e[i])
    n = len(uniq)
    if n < p["min_eigenvalue_size"]:
        return np.float32(-1)
    chi, count = np.float32(0), 0
    bins = p["histogram_bin_size"]
    w = np.float32(np.float32(3.0) / np.float32(bins))
    for pace in range(p["min_unfolding_pace"], p["max_unfolding_pace"] + 1):
        if n // pace < 5:
            break
        ns = n // pace
        xs = np.array([float(uniq[i * pace]) for i in range(ns)])
        ys = np.array([(i * pace + 1) / n for i in range(ns)])
        xs[-1] = float(uniq[-1])
        ys[-1] = 1.0
        if np.any(np.diff(xs) <= 0):
            raise RMTSplineError(f"unfolding at pace {pace}: eigenvalues not increasing in |lambda| order")
        spline = Akima1DInterpolator(xs, ys)
        se = np.zeros(n, np.float32)
        se[-1] = 1.0
        se[1:-1] = spline(np.array([float(v) for v in uniq[1:-1]])).astype(np.float32)
        spacings = (se[1:] - se[:-1]) * np.float32(n)
        hist = np.zeros(bins, np.float32)
        for s in spacings:
            if np.float32(0) <= s < np.float32(3):
                b = int(np.float32(s / w))
                if b < bins:
                    hist[b] += 1
        c = np.float32(0)
        for i in range(bins):
            E = np.float32((np.exp(np.float32(-i * w)) - np.exp(np.float32(-(i + 1) * w))) * np.float32(n))
            c = np.float32(c + np.float32((hist[i] - E) * (hist[i] - E)) / E)
        chi = np.float32(chi + c)
        count += 1
    return np.float32(chi / np.float32(count))


def rmt_run(G, K, x, y, c, r, **kw):
    """RMT::process: returns (threshold or None when no threshold above tstop passes, steps)."""
    p = dict(RMT_DEFAULTS)
    p.update(kw)
    mat = rmt_dense(G, K, np.asarray(x), np.asarray(y), np.asarray(c), np.asarray(r, np.float32))
    maxs = rmt_maximums(mat)
    final_t, final_chi, max_chi = np.float32(0), np.float32(np.inf), np.float32(-np.inf)
    t = np.float32(p["threshold_start"])
    steps = []
    while max_chi < np.float32(p["chi_square_threshold2"]):
        e = rmt_prune_eigenvalues(mat, maxs, t)
        chi = np.float32(-1)
        if len(e) > 0:
            chi = rmt_chi_square(e, p)
        if chi != np.float32(-1):
            if chi < np.float32(p["chi_square_threshold1"]):
                final_chi, final_t = chi, t
            if final_chi < np.float32(p["chi_square_threshold1"]) and chi > final_chi:
                max_chi = chi
        steps.append((float(t), len(e), float(chi)))
        t = np.float32(t - np.float32(p["threshold_step"]))
        if t < np.float32(p["threshold_stop"]):
            return None, steps
    return float(final_t), steps
