"""ctypes bindings for the CPU checkers (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this module.  It wraps:

* the C restatement (``libkinc_oracle.so``, built from kinc_oracle.c), and
* KINC's own Pairwise:: sources compiled by build_ref.py
  (``oracle/_ref/libkinc_ref{0,1,2}.so``), when the KINC tree was available
  to build them.
"""
import ctypes
import ctypes.util
import math
import os
import re

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


class KoclParams(ctypes.Structure):
    _fields_ = [("clus_method", ctypes.c_int32), ("corr_method", ctypes.c_int32), ("min_expr", ctypes.c_float),
                ("min_samples", ctypes.c_int32), ("min_clusters", ctypes.c_int32), ("max_clusters", ctypes.c_int32),
                ("criterion", ctypes.c_int32), ("pre_out", ctypes.c_int32), ("post_out", ctypes.c_int32),
                ("ksize", ctypes.c_int32)]


_ocl = []


def ocl_lib():
    """KINC's OpenCL kernels compiled for the host and driven like its OpenCL worker, or None
    when the KINC tree is absent."""
    if not _ocl:
        path = build_ref.build_ocl()
        L = None
        if path is not None:
            L = ctypes.CDLL(path)
            L.kocl_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(KoclParams),
                                   ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]
            L.kocl_run.restype = ctypes.c_int
        _ocl.append(L)
    return _ocl[0]


def run_ocl(gem, p, start, size, ksize=4096):
    """The OpenCL worker's results for pairs [start, start+size) (K, labels, corr), computed by
    KINC's own OpenCL kernels on the CPU; None when they are not built.  `p` is a KoParams
    (clustering none or GMM)."""
    L = ocl_lib()
    if L is None:
        return None
    gem = np.ascontiguousarray(gem, dtype=np.float32)
    G, S = gem.shape
    q = KoclParams(p.clus_method, p.corr_method, p.min_expr, p.min_samples, p.min_clusters, p.max_clusters,
                   p.criterion, p.pre_out, p.post_out, ksize)
    K = np.zeros(size, np.int8)
    labels = np.zeros((size, S), np.int8)
    corr = np.zeros((size, p.max_clusters), np.float32)
    if L.kocl_run(_ptr(gem), G, S, ctypes.byref(q), start, size, _ptr(K), _ptr(labels), _ptr(corr)) != 0:
        raise ValueError("the OpenCL worker would not run these arguments")
    return K, labels, corr


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
    corr = np.zeros((size, p.max_clusters, 2) if p.corr_method == 2 else (size, p.max_clusters), np.float32)
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
    corr = np.zeros((n, p.max_clusters, 2) if p.corr_method == 2 else (n, p.max_clusters), np.float32)
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


# ----------------------------------------------------------------------------- text import / export
# The text analytics restated over Python strings: QTextStream's readLine + split on white
# space, QString::toInt / toDouble / toFloat in the C locale, and the number formats of the
# writers.  Parse failures raise TextError.

class TextError(ValueError):
    """A line the reference's import rejects; .order is True for a pair out of increasing order."""

    def __init__(self, msg, order=False):
        super().__init__(msg)
        self.order = order


_NUMBER = re.compile(r"(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")
_INT = re.compile(r"[+-]?\d+")
_SPACE = re.compile(r"[ \t\n\r\v\f]+")


def _fields(line):
    """The line split on ASCII white space, empty parts dropped."""
    return [w for w in _SPACE.split(line) if w]


def qt_to_double(w):
    """QString::toDouble: a float, or None when the field is not a number (overflow and
    underflow to zero included)."""
    sign, body = (w[0], w[1:]) if w[:1] in ("+", "-") else ("", w)
    if body.lower() == "inf":
        return -math.inf if sign == "-" else math.inf
    if not sign and body.lower() == "nan":
        return math.nan
    m = _NUMBER.fullmatch(body)
    if not m:
        return None
    v = float(body)
    if math.isinf(v) or (v == 0.0 and any(ch in "123456789" for ch in m.group(1))):
        return None
    return -v if sign == "-" else v


def qt_to_int(w):
    """QString::toInt: 0 unless the field is an int."""
    if not _INT.fullmatch(w):
        return 0
    v = int(w)
    return v if -2**31 <= v < 2**31 else 0


_libm = None


def _libm_float(name):
    """The C library's float function `name` (logf, expf, ...), which the reference's calls on a
    float value resolve to."""
    global _libm
    if _libm is None:
        _libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    f = getattr(_libm, name)
    f.restype, f.argtypes = ctypes.c_float, [ctypes.c_float]
    return f


def _transform_value(v, transform):
    """ImportExpressionMatrix's transform of the float value (src/core/importexpressionmatrix.cpp:
    108-123): log, log2, log10 of a float."""
    v = np.float32(v)
    if transform in (1, 2, 3):
        return np.float32(_libm_float(("logf", "log2f", "log10f")[transform - 1])(float(v)))
    return v


def import_emx_text(text, nan=None, samples=0, transform=0):
    """ImportExpressionMatrix::process restated (src/core/importexpressionmatrix.cpp:20-180);
    returns (gem float32 [genes][samples], gene names, sample names).  Lines without fields are
    skipped."""
    S = samples
    sample_names = [str(i) for i in range(S)]
    gene_names, rows = [], []
    for line in text.split("\n"):
        w = _fields(line)
        if not w:
            continue
        if S == 0:
            S = len(w)
            sample_names = list(w)
            continue
        if len(w) != S + 1:
            raise TextError(f"Encountered gene expression line with incorrect amount of fields. Read in {len(w) - 1} "
                            f"fields when it should have been {S}. Gene name is {w[0]}.")
        row = []
        for tok in w[1:]:
            if nan and tok == nan:
                row.append(np.float32(math.nan))
                continue
            d = qt_to_double(tok)
            if d is None:
                raise TextError(f'Failed to read expression value "{tok}" for gene {w[0]}.')
            row.append(_transform_value(d, transform))
        gene_names.append(w[0])
        rows.append(row)
    return np.array(rows, np.float32).reshape(len(rows), S), gene_names, sample_names


def export_emx_text(gem, gene_names=None, sample_names=None, transform=0, nan=None):
    """ExportExpressionMatrix::process restated (src/core/exportexpressionmatrix.cpp:20-100): the
    transform undone on the float (exp of a float; pow(2 or 10, v) in double, rounded to float),
    printed at 12 significant digits."""
    G, S = gem.shape
    gene_names = [str(g) for g in range(G)] if gene_names is None else gene_names
    sample_names = [str(s) for s in range(S)] if sample_names is None else sample_names
    out = ["".join(f"{n}\t" for n in sample_names), "\n"]
    for g in range(G):
        out.append(gene_names[g])
        for s in range(S):
            v = np.float32(gem[g, s])
            if np.isnan(v):
                out.append("\t" + (nan or ""))
                continue
            if transform == 1:
                v = np.float32(_libm_float("expf")(float(v)))
            elif transform == 2:
                v = np.float32(math.pow(2.0, float(v)))
            elif transform == 3:
                v = np.float32(math.pow(10.0, float(v)))
            out.append("\t%.12g" % float(v))
        out.append("\n")
    return "".join(out)


def import_cmx_text(text, genes, max_clusters, samples):
    """ImportCorrelationMatrix::process restated (src/core/importcorrelationmatrix.cpp:22-141) as
    its loop intends: consecutive lines of one pair are its clusters, numbered in line order; the
    pair is written once (CMX always, CCM when it has more than one cluster); lines of 0 or 1
    fields are skipped.  Returns (ccm, cmx) item dicts like pairwise_matrix.read's."""
    ccm = dict(x=[], y=[], c=[], payload=[])
    cmx = dict(x=[], y=[], c=[], payload=[])
    pending, cur, last = [], None, -1

    def close():
        for k, (r, codes) in enumerate(pending):
            cmx["x"].append(cur[0]), cmx["y"].append(cur[1]), cmx["c"].append(k), cmx["payload"].append([r])
            if len(pending) > 1:
                ccm["x"].append(cur[0]), ccm["y"].append(cur[1]), ccm["c"].append(k), ccm["payload"].append(codes)
        pending.clear()

    for line in text.split("\n"):
        w = _fields(line)
        if len(w) <= 1:
            continue
        if len(w) != 11:
            raise TextError(f"Encountered line with incorrect amount of fields. Read {len(w)} fields when there "
                            f"should have been 11.")
        x, y = qt_to_int(w[0]), qt_to_int(w[1])
        d = qt_to_double(w[9])
        r = np.float32(0.0 if d is None else d)
        mask = w[10]
        if len(mask) != samples:
            raise TextError(f"Encountered sample mask with invalid length {len(mask)}. Sample size is {samples}.")
        if x < 1 or y < 0 or x <= y or x >= genes:
            raise TextError(f"Cannot initialize pairwise index ({x}, {y}).")
        if not pending or (x, y) != cur:
            p = x * (x - 1) // 2 + y
            if p <= last:
                raise TextError(f"pair ({x}, {y}) out of order", order=True)
            close()
            cur, last = (x, y), p
        if len(pending) + 1 > max_clusters:
            raise TextError(f"Cannot write pair with cluster size {len(pending) + 1} exceeding the max of "
                            f"{max_clusters}.")
        pending.append((r, [int(ch) if "0" <= ch <= "9" else -1 for ch in mask]))
    close()
    for d, dt in ((ccm, np.int8), (cmx, np.float32)):
        for key in ("x", "y"):
            d[key] = np.array(d[key], np.int32)
        d["c"] = np.array(d["c"], np.int8)
        d["payload"] = np.array(d["payload"], dt).reshape(len(d["c"]), samples if dt is np.int8 else 1)
    return ccm, cmx


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
