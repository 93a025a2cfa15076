"""Host-side mirror of KINC's Similarity analytic over the GB300 worker.

Same argument names, defaults and meanings as the reference's CLI
(src/core/similarity_input.cpp:96-254, defaults src/core/similarity.h:58-71),
same block split (src/core/similarity.cpp:17-39), same per-block result
(src/core/similarity_resultblock.h:7-23) and the same ordered CCM/CMX
emission (src/core/similarity.cpp:66-127).  The per-pair work runs in
libkinc_gb300.so through the C ABI in include/kinc_sim.h; this module only
marshals arguments and arrays.
"""
import ctypes
import math
from dataclasses import dataclass

import numpy as np

from . import _native

CLUSTERING_NAMES = ["none", "gmm", "kmeans"]
CORRELATION_NAMES = ["pearson", "spearman", "both"]
CRITERION_NAMES = ["BIC", "ICL"]
SEMANTICS_NAMES = ["reference", "fixed"]
RAND_NAMES = ["glibc", "lcg"]
PRECISION_NAMES = ["fp32", "tf32", "3xbf16", "fp32tiled", "fp16"]


class InvalidArgument(ValueError):
    """Raised where the reference throws E_MAKE_EXCEPTION "Invalid Argument"."""


@dataclass
class WorkBlock:
    index: int
    start: int
    size: int


@dataclass
class ResultBlock:
    index: int
    start: int
    K: np.ndarray          # int8 [size]
    labels: np.ndarray     # int8 [size, samples]
    corr: np.ndarray       # float32 [size, maxclus] ([size, maxclus, 2] with corrmethod both)


def _choice(value, names, what):
    if isinstance(value, (int, np.integer)):
        if 0 <= int(value) < len(names):
            return int(value)
    elif value in names:
        return names.index(value)
    elif isinstance(value, str) and value.lower() in [n.lower() for n in names]:
        return [n.lower() for n in names].index(value.lower())
    raise InvalidArgument(f"{what} must be one of {names}, got {value!r}")


class PairwiseMatrix:
    """In-memory CCM or CMX item list written in strictly increasing
    indent = (x(x-1)/2 + y) * 64 + cluster order (src/core/pairwise_matrix.cpp:122-151)."""

    MAX_CLUSTER_SIZE = 64

    def __init__(self, kind, genes, max_clusters, samples):
        self.kind = kind
        self.genes = genes
        self.max_clusters = max_clusters
        self.samples = samples
        self.x, self.y, self.c, self.data = [], [], [], []
        self.pairs = 0
        self._last = -1

    def write_pair(self, x, y, clusters):
        """Matrix::Pair::write (src/core/pairwise_matrix.cpp:251-273)."""
        if len(clusters) > self.max_clusters:
            raise ValueError(f"Cannot write pair with cluster size {len(clusters)} exceeding the max of "
                             f"{self.max_clusters}.")
        base = (x * (x - 1) // 2 + y) * self.MAX_CLUSTER_SIZE
        for i, payload in enumerate(clusters):
            indent = base + i
            if indent <= self._last:
                raise ValueError(f"Attempting to write indent {base} when last written is {self._last}.")
            self.x.append(x)
            self.y.append(y)
            self.c.append(i)
            self.data.append(payload)
            self._last = indent
        self.pairs += 1

    def __len__(self):
        return len(self.x)

    def arrays(self):
        x = np.asarray(self.x, np.int32)
        y = np.asarray(self.y, np.int32)
        c = np.asarray(self.c, np.int8)
        if self.kind == "cmx":
            return x, y, c, np.asarray(self.data, np.float32).reshape(-1)
        return x, y, c, np.asarray(self.data, np.int8).reshape(len(self.x), self.samples)


class Similarity:
    """KINC Similarity analytic on the GB300 worker.

    Beyond KINC's arguments: semantics ("reference": KINC's serial path including its
    packed-array reads in Pearson/Spearman; "fixed": each sample's own values), rand
    ("glibc": the serial path's process-global rand() stream; "lcg": the OpenCL worker's GMM,
    with its per-fit LCG, float BIC/ICL and zero-determinant failure rule) and precision
    (tensor-core forms of pairwise-complete Pearson)."""

    WORK_BLOCK_SIZE = _native.WORK_BLOCK_SIZE

    def __init__(self, expressions, clusmethod="none", corrmethod="pearson", minexpr=-math.inf, minsamp=30,
                 minclus=1, maxclus=5, crit="ICL", preout=False, postout=False, mincorr=0.5, maxcorr=1.0,
                 ksize=4096, semantics="reference", rand="glibc", precision="fp32"):
        self.expressions = np.ascontiguousarray(expressions, dtype=np.float32)
        if self.expressions.ndim != 2:
            raise InvalidArgument("Did not get valid input and/or output arguments.")
        self.params = _native.SimParams()
        _native.load().kinc_sim_params_default(ctypes.byref(self.params))
        p = self.params
        p.clus_method = _choice(clusmethod, CLUSTERING_NAMES, "clusmethod")
        p.corr_method = _choice(corrmethod, CORRELATION_NAMES, "corrmethod")
        p.min_expr = float(minexpr)
        p.min_samples = int(minsamp)
        p.min_clusters = int(minclus)
        p.max_clusters = int(maxclus)
        p.criterion = _choice(crit, CRITERION_NAMES, "crit")
        p.pre_out = int(bool(preout))
        p.post_out = int(bool(postout))
        p.min_corr = float(mincorr)
        p.max_corr = float(maxcorr)
        p.ksize = int(ksize)
        p.semantics = _choice(semantics, SEMANTICS_NAMES, "semantics")
        p.rand_mode = _choice(rand, RAND_NAMES, "rand")
        p.precision = _choice(precision, PRECISION_NAMES, "precision")
        self._ctx = None
        self.ccm = None
        self.cmx = None

    # -- EAbstractAnalytic ------------------------------------------------
    @property
    def genes(self):
        return self.expressions.shape[0]

    @property
    def samples(self):
        return self.expressions.shape[1]

    def initialize(self):
        """Similarity::initialize (src/core/similarity.cpp:164-197) + worker creation."""
        p = self.params
        if p.max_clusters < p.min_clusters:
            raise InvalidArgument("Minimum clusters must be less than or equal to maximum clusters.")
        if self._ctx is None:
            L = _native.load()
            ctx = ctypes.c_void_p()
            rc = L.kinc_sim_create(self.expressions.ctypes.data_as(ctypes.c_void_p), self.genes, self.samples,
                                   ctypes.byref(p), ctypes.byref(ctx))
            if rc == _native.EINVAL:
                raise InvalidArgument(L.kinc_sim_last_error(None).decode())
            _native.check(rc, None)
            self._ctx = ctx
        self.ccm = PairwiseMatrix("ccm", self.genes, p.max_clusters, self.samples)
        self.cmx = PairwiseMatrix("cmx", self.genes, p.max_clusters, self.samples)

    def launch(self):
        """The per-pair kernel's launch shape (kinc_sim_get_launch) as a dict."""
        if self._ctx is None:
            self.initialize()
        L = _native.load()
        out = _native.Launch()
        _native.check(L.kinc_sim_get_launch(self._ctx, ctypes.byref(out)), self._ctx)
        return out.as_dict()

    def set_launch(self, warps_per_cta, rounds, prefetch):
        """Fix the launch shape (kinc_sim_set_launch); every shape gives the same results."""
        if self._ctx is None:
            self.initialize()
        L = _native.load()
        _native.check(L.kinc_sim_set_launch(self._ctx, ctypes.byref(_native.Launch(warps_per_cta, rounds, prefetch,
                                                                                       0))), self._ctx)

    def autotune(self, start=None, size=None, use_cache=True, cap=64):
        """Pick the launch shape by timing candidates on pairs [start, start+size)
        (kinc_sim_autotune; default: 311,296 pairs from the middle -- 4 tiles of 32 pairs for each
        warp of 16-warp CTAs on 152 SMs -- at most one device block).  Returns (chosen shape, timed
        candidates)."""
        if self._ctx is None:
            self.initialize()
        L = _native.load()
        total = self.total_pairs()
        if size is None:
            size = 4 * 32 * 16 * 152
        size = int(min(size, total, L.kinc_sim_max_device_block(self._ctx)))
        if start is None:
            start = max(0, total // 2 - size // 2)
        chosen = _native.Launch()
        entries = (_native.TuneEntry * cap)()
        n = ctypes.c_int32(0)
        _native.check(L.kinc_sim_autotune(self._ctx, int(start), size, int(bool(use_cache)), ctypes.byref(chosen),
                                          entries, cap, ctypes.byref(n)), self._ctx)
        timed = [dict(entries[i].launch.as_dict(), ms=entries[i].ms) for i in range(min(n.value, cap))]
        return chosen.as_dict(), timed

    def close(self):
        if self._ctx is not None:
            _native.load().kinc_sim_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def total_pairs(self):
        return self.genes * (self.genes - 1) // 2

    def size(self):
        """Similarity::size (src/core/similarity.cpp:17-23)."""
        return (self.total_pairs() + self.WORK_BLOCK_SIZE - 1) // self.WORK_BLOCK_SIZE

    def make_work(self, index):
        """Similarity::makeWork (src/core/similarity.cpp:30-39)."""
        start = index * self.WORK_BLOCK_SIZE
        return WorkBlock(index, start, min(self.total_pairs() - start, self.WORK_BLOCK_SIZE))

    def execute(self, work, start=None, size=None):
        """Worker::execute: one work block -> one result block (host arrays)."""
        if self._ctx is None:
            self.initialize()
        if isinstance(work, WorkBlock):
            index, start, size = work.index, work.start, work.size
        else:
            index = -1
        S, maxk = self.samples, self.params.max_clusters
        K = np.empty(size, np.int8)
        labels = np.empty((size, S), np.int8)
        corr = np.empty((size, maxk, 2) if self.params.corr_method == 2 else (size, maxk), np.float32)
        rc = _native.load().kinc_sim_execute_block(self._ctx, start, size, K.ctypes.data_as(ctypes.c_void_p),
                                                   labels.ctypes.data_as(ctypes.c_void_p),
                                                   corr.ctypes.data_as(ctypes.c_void_p))
        _native.check(rc, self._ctx)
        return ResultBlock(index, start, K, labels, corr)

    def process(self, result):
        """Similarity::process (src/core/similarity.cpp:66-127) via the native filter."""
        L = _native.load()
        size = len(result.K)
        S, maxk = self.samples, self.params.max_clusters
        nc = 2 if self.params.corr_method == 2 else 1
        cap = max(1, size * maxk)
        cx, cy, cc, cr = (np.empty(cap, np.int32), np.empty(cap, np.int32), np.empty(cap, np.int8),
                          np.empty((cap, nc), np.float32))
        mx, my, mc = np.empty(cap, np.int32), np.empty(cap, np.int32), np.empty(cap, np.int8)
        codes = np.empty((cap, S), np.int8)
        n_cmx, n_ccm = ctypes.c_int64(0), ctypes.c_int64(0)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        rc = L.kinc_sim_process_block(self._ctx, result.start, size, vp(result.K), vp(result.labels),
                                      vp(result.corr), vp(cx), vp(cy), vp(cc), vp(cr), cap, ctypes.byref(n_cmx),
                                      vp(mx), vp(my), vp(mc), vp(codes), cap, ctypes.byref(n_ccm))
        _native.check(rc, self._ctx)
        self._append(self.cmx, cx[:n_cmx.value], cy[:n_cmx.value], cc[:n_cmx.value],
                     list(cr[:n_cmx.value, 0]) if nc == 1 else [tuple(r) for r in cr[:n_cmx.value]])
        self._append(self.ccm, mx[:n_ccm.value], my[:n_ccm.value], mc[:n_ccm.value],
                     [codes[i] for i in range(n_ccm.value)])

    @staticmethod
    def _append(matrix, x, y, c, payloads):
        i = 0
        n = len(x)
        while i < n:
            j = i
            while j < n and x[j] == x[i] and y[j] == y[i]:
                j += 1
            matrix.write_pair(int(x[i]), int(y[i]), payloads[i:j])
            i = j

    def run(self, ccm_path=None, cmx_path=None, little_endian=False, first_block=0, nblocks=-1, device_block=0,
            world=None, rank=0, by_cost=False, resume=False):
        """Run work blocks [first_block, first_block + nblocks) in order (all of them by default),
        or, with `world`, the share of rank `rank` (kinc_shard_blocks: equal block counts, or equal
        estimated cost with by_cost).  With file paths, the native runner writes the CCM/CMX files
        (include/kinc_pairwise_matrix.h) in device blocks of `device_block` pairs (0 = the largest
        the worker holds); with resume, files an interrupted run left are cut back to their whole
        work blocks and only the rest is run and appended.  Without file paths the items are kept
        in memory and (ccm, cmx) PairwiseMatrix objects are returned."""
        if world is not None:
            from .shard import shard_blocks
            if first_block or nblocks != -1:
                raise InvalidArgument("give world/rank or first_block/nblocks, not both")
            first_block, nblocks = shard_blocks(self.expressions, world, rank, by_cost=by_cost,
                                                min_expr=self.params.min_expr)
        if ccm_path is not None or cmx_path is not None:
            if resume:
                self._resume_to_files(ccm_path, cmx_path, little_endian, first_block, nblocks, device_block)
            else:
                self._run_to_files(ccm_path, cmx_path, little_endian, first_block, nblocks, device_block)
            return ccm_path, cmx_path
        self.initialize()
        last = self.size() if nblocks < 0 else min(self.size(), first_block + nblocks)
        for b in range(first_block, last):
            self.process(self.execute(self.make_work(b)))
        return self.ccm, self.cmx

    def _run_to_files(self, ccm_path, cmx_path, little_endian, first_block, nblocks, device_block):
        """kinc_sim_run_to_files_ex: blocks [first_block, first_block + nblocks) into new files."""
        self.initialize()
        L = _native.load()
        rc = L.kinc_sim_run_to_files_ex(self._ctx, str(ccm_path).encode() if ccm_path else None,
                                        str(cmx_path).encode() if cmx_path else None, int(little_endian),
                                        int(first_block), int(nblocks), int(device_block))
        if rc != _native.OK:
            raise _native.SimError(rc, L.kinc_pm_last_error().decode())

    def _resume_to_files(self, ccm_path, cmx_path, little_endian, first_block, nblocks, device_block):
        """Cut the files back to their whole work blocks (kinc_pm_resume_point), run the remaining
        blocks into part files and join them after the kept items (kinc_pm_concat)."""
        import os

        from . import pairwise_matrix as pm
        end = self.size() if nblocks < 0 else min(self.size(), first_block + nblocks)
        start = pm.resume_point(ccm_path, cmx_path, first_block=first_block, little_endian=little_endian)
        if start > end:
            raise InvalidArgument(f"the files hold work blocks past block {end}: not an interrupted run of "
                                  f"these blocks")
        finals = [str(p) for p in (ccm_path, cmx_path) if p is not None]
        parts = {f: f + ".part" for f in finals}
        self._run_to_files(parts.get(str(ccm_path)) if ccm_path is not None else None,
                           parts.get(str(cmx_path)) if cmx_path is not None else None,
                           little_endian, start, end - start, device_block)
        for final, part in parts.items():
            if os.path.exists(final):
                pm.concat(final + ".joined", [final, part], little_endian=little_endian)
                os.replace(final + ".joined", final)
                os.remove(part)
            else:
                os.replace(part, final)
