"""Host-side mirror of KINC's RMT analytic over the GB300 library.

Same argument names, defaults and checks as the reference's CLI
(src/core/rmt_input.cpp:51-140: input, log, tstart, tstep, tstop, minpace,
maxpace, bins; defaults src/core/rmt.h:31-39) and the same result: the
correlation threshold above which the correlation matrix's eigenvalue
spacings stop looking random (src/core/rmt.cpp:33-122).  The work runs in
libkinc_gb300.so through include/kinc_rmt.h.
"""
import ctypes

import numpy as np

from . import _native


class RMT:
    """KINC RMT analytic on the GPU."""

    def __init__(self, tstart=0.99, tstep=0.001, tstop=0.5, minpace=10, maxpace=40, bins=60,
                 chi1=99.607, chi2=200.0, mineigens=50):
        self.params = _native.RmtParams()
        _native.load().kinc_rmt_params_default(ctypes.byref(self.params))
        p = self.params
        p.threshold_start, p.threshold_step, p.threshold_stop = float(tstart), float(tstep), float(tstop)
        p.min_unfolding_pace, p.max_unfolding_pace, p.histogram_bin_size = int(minpace), int(maxpace), int(bins)
        p.chi_square_threshold1, p.chi_square_threshold2 = float(chi1), float(chi2)
        p.min_eigenvalue_size = int(mineigens)

    def _check(self, rc):
        if rc != _native.OK:
            raise _native.SimError(rc, _native.load().kinc_rmt_last_error().decode())

    def run(self, input=None, log=None, items=None, genes=None, max_clusters=None, little_endian=False,
            max_steps=4096, strict=True):
        """The threshold for a CMX file (`input`) or for items (x, y, c, r) of a `genes` x `max_clusters`
        matrix; returns (threshold, steps) with steps an array of (threshold, size, chi) rows.  When no
        threshold above tstop passes, raises (the reference's error) unless `strict` is false, which
        returns (None, steps) for items."""
        L = _native.load()
        out = ctypes.c_float(0)
        log_b = str(log).encode() if log is not None else None
        if input is not None:
            self._check(L.kinc_rmt_run(str(input).encode(), int(little_endian), ctypes.byref(self.params), log_b,
                                       ctypes.byref(out)))
            return float(out.value), None
        x, y, c, r = (np.ascontiguousarray(a, t) for a, t in zip(items, (np.int32, np.int32, np.int8, np.float32)))
        steps = np.zeros((max_steps, 3), np.float32)
        nsteps = ctypes.c_int32(0)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        rc = L.kinc_rmt_run_items(int(genes), int(max_clusters), len(x), vp(x), vp(y), vp(c), vp(r),
                                  ctypes.byref(self.params), log_b, ctypes.byref(out), vp(steps), max_steps,
                                  ctypes.byref(nsteps))
        if rc == _native.RMT_ENOTHRESHOLD and not strict:
            return None, steps[:min(nsteps.value, max_steps)]
        self._check(rc)
        return float(out.value), steps[:min(nsteps.value, max_steps)]

    def prune_eigenvalues(self, items, genes, max_clusters, threshold):
        """Eigenvalues of the pruned matrix at one threshold, ascending |lambda| (float)."""
        L = _native.load()
        x, y, c, r = (np.ascontiguousarray(a, t) for a, t in zip(items, (np.int32, np.int32, np.int8, np.float32)))
        out = np.zeros(int(genes) * int(max_clusters), np.float32)
        m = ctypes.c_int32(0)
        vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        self._check(L.kinc_rmt_prune_eigenvalues(int(genes), int(max_clusters), len(x), vp(x), vp(y), vp(c), vp(r),
                                                 ctypes.c_float(threshold), vp(out), ctypes.byref(m)))
        return out[:m.value]

    def chi_square(self, eigens):
        """computeChiSquare on eigenvalues sorted by ascending |lambda|: -1 with too few unique values."""
        e = np.ascontiguousarray(eigens, np.float32)
        chi = ctypes.c_float(0)
        self._check(_native.load().kinc_rmt_chi_square(e.ctypes.data_as(ctypes.c_void_p), len(e),
                                                       ctypes.byref(self.params), ctypes.byref(chi)))
        return float(chi.value)
