"""KINC's pairwise matrix files (CCM cluster matrix, CMX correlation matrix)
and expression matrix (EMX) data section, read and written by the native
library (include/kinc_pairwise_matrix.h)."""
import ctypes

import numpy as np

from . import _native

CCM, CMX = 1, 2


def _check(rc):
    if rc != _native.OK:
        raise _native.SimError(rc, _native.load().kinc_pm_last_error().decode())


def write(path, kind, genes, max_clusters, subsize, x, y, c, payload, little_endian=False):
    """Write a CCM (payload int8 codes [n][samples]) or CMX (payload float32 [n][subsize]) file."""
    L = _native.load()
    h = ctypes.c_void_p()
    _check(L.kinc_pm_create(str(path).encode(), kind, genes, max_clusters, subsize, int(little_endian),
                            ctypes.byref(h)))
    try:
        x = np.ascontiguousarray(x, np.int32)
        y = np.ascontiguousarray(y, np.int32)
        c = np.ascontiguousarray(c, np.int8)
        payload = np.ascontiguousarray(payload, np.int8 if kind == CCM else np.float32)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        _check(L.kinc_pm_write_items(h, len(x), vp(x), vp(y), vp(c), vp(payload)))
    finally:
        _check(L.kinc_pm_close(h))


def read(path, kind, little_endian=False):
    """Read a CCM/CMX file: dict(genes, max_clusters, subsize, pairs, x, y, c, payload)."""
    L = _native.load()
    h = ctypes.c_void_p()
    g, k, s = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    pairs, clusters = ctypes.c_int64(), ctypes.c_int64()
    _check(L.kinc_pm_open(str(path).encode(), kind, int(little_endian), ctypes.byref(h), ctypes.byref(g),
                          ctypes.byref(k), ctypes.byref(s), ctypes.byref(pairs), ctypes.byref(clusters)))
    try:
        n = clusters.value
        x = np.empty(n, np.int32)
        y = np.empty(n, np.int32)
        c = np.empty(n, np.int8)
        payload = np.empty((n, s.value), np.int8 if kind == CCM else np.float32)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        _check(L.kinc_pm_read_items(h, 0, n, vp(x), vp(y), vp(c), vp(payload)))
    finally:
        L.kinc_pm_close(h)
    return dict(genes=g.value, max_clusters=k.value, subsize=s.value, pairs=pairs.value, x=x, y=y, c=c,
                payload=payload)


def write_emx(path, gem, little_endian=False):
    gem = np.ascontiguousarray(gem, np.float32)
    _check(_native.load().kinc_emx_write(str(path).encode(), gem.ctypes.data_as(ctypes.c_void_p), gem.shape[0],
                                         gem.shape[1], int(little_endian)))


def read_emx(path, little_endian=False):
    L = _native.load()
    g, s = ctypes.c_int32(), ctypes.c_int32()
    _check(L.kinc_emx_read_header(str(path).encode(), int(little_endian), ctypes.byref(g), ctypes.byref(s)))
    gem = np.empty((g.value, s.value), np.float32)
    _check(L.kinc_emx_read(str(path).encode(), int(little_endian), gem.ctypes.data_as(ctypes.c_void_p), gem.size))
    return gem


def resume_point(ccm_path, cmx_path, first_block=0, little_endian=False):
    """Cut an interrupted run's CCM/CMX files back to their finished work blocks; returns the
    block to resume from (include/kinc_pairwise_matrix.h: kinc_pm_resume_point)."""
    enc = lambda p: str(p).encode() if p is not None else None  # noqa: E731
    r = ctypes.c_int64()
    _check(_native.load().kinc_pm_resume_point(enc(ccm_path), enc(cmx_path), int(little_endian), int(first_block),
                                               ctypes.byref(r)))
    return r.value


def concat(out_path, in_paths, little_endian=False):
    """The CCM or CMX files of a sharded run joined into one, in rank order."""
    arr = (ctypes.c_char_p * len(in_paths))(*[str(p).encode() for p in in_paths])
    _check(_native.load().kinc_pm_concat(str(out_path).encode(), arr, len(in_paths), int(little_endian)))


def export_text(ccm_path, cmx_path, out_path, little_endian=False):
    """ExportCorrelationMatrix: the CMX/CCM pair as tab-separated text (one line per CMX cluster)."""
    _check(_native.load().kinc_pm_export_text(str(ccm_path).encode(), str(cmx_path).encode(), int(little_endian),
                                              str(out_path).encode()))


def extract(emx_path, ccm_path, cmx_path, tsv_path=None, graphml_path=None, names_path=None, min_corr=0.85,
            max_corr=1.0, little_endian=False):
    """Extract: the network of clusters with min_corr <= |r| <= max_corr as TSV and/or GraphML."""
    enc = lambda p: str(p).encode() if p is not None else None  # noqa: E731
    _check(_native.load().kinc_pm_extract(enc(emx_path), enc(ccm_path), enc(cmx_path), enc(names_path),
                                          int(little_endian), float(min_corr), float(max_corr), enc(tsv_path),
                                          enc(graphml_path)))


def import_text(in_path, ccm_path, cmx_path, genes, max_clusters, samples, little_endian=False):
    """ImportCorrelationMatrix: 11-column text (as export_text writes it) -> CCM + CMX files."""
    _check(_native.load().kinc_pm_import_text(str(in_path).encode(), str(ccm_path).encode(), str(cmx_path).encode(),
                                              int(genes), int(max_clusters), int(samples), int(little_endian)))


# ExpressionMatrix::TRANSFORM_NAMES (src/core/expressionmatrix.cpp:8-14), in their enum order
TRANSFORMS = ("none", "natural logarithm", "logarithm base 2", "logarithm base 10")


def _transform(t):
    if isinstance(t, int):
        if not 0 <= t < len(TRANSFORMS):
            raise ValueError(f"transform {t} is not one of 0..{len(TRANSFORMS) - 1}")
        return t
    names = [n.lower() for n in TRANSFORMS]
    if str(t).lower() not in names:
        raise ValueError(f"transform must be one of {', '.join(TRANSFORMS)}")
    return names.index(str(t).lower())


def import_emx_text(in_path, emx_path, nan=None, samples=0, transform="none", gene_names_path=None,
                    sample_names_path=None, little_endian=False):
    """ImportExpressionMatrix: text (gene name + one value per sample per line; with samples=0 the
    first line names the samples) -> EMX; the names go one per line to the *_names_path files."""
    enc = lambda p: str(p).encode() if p is not None else None  # noqa: E731
    _check(_native.load().kinc_emx_import_text(enc(in_path), enc(nan), int(samples), _transform(transform),
                                               int(little_endian), enc(emx_path), enc(gene_names_path),
                                               enc(sample_names_path)))


def export_emx_text(emx_path, out_path, nan=None, transform="none", gene_names_path=None, sample_names_path=None,
                    little_endian=False):
    """ExportExpressionMatrix: EMX -> text, undoing the transform the matrix was imported with."""
    enc = lambda p: str(p).encode() if p is not None else None  # noqa: E731
    _check(_native.load().kinc_emx_export_text(enc(emx_path), int(little_endian), enc(gene_names_path),
                                               enc(sample_names_path), _transform(transform), enc(nan),
                                               enc(out_path)))
