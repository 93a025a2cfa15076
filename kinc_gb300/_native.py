"""ctypes binding of libkinc_gb300.so (include/kinc_sim.h).

There is no CPU fallback: if the library is missing or cannot be loaded,
every entry point raises.  On a machine without a GPU the library still
loads (the CUDA runtime is linked dynamically), so symbol checks work, but
kinc_sim_create fails with a CUDA error.
"""
import ctypes
import os

from . import build as _build

_lib = None

OK, EINVAL, ECUDA, ENOMEM, EKERNEL, EORDER, EIO = 0, 1, 2, 3, 4, 5, 8
WORK_BLOCK_SIZE = 32768


class SimParams(ctypes.Structure):
    """kinc_sim_params (include/kinc_sim.h)."""
    _fields_ = [("clus_method", ctypes.c_int32), ("corr_method", ctypes.c_int32),
                ("min_expr", ctypes.c_float), ("min_samples", ctypes.c_int32),
                ("min_clusters", ctypes.c_int32), ("max_clusters", ctypes.c_int32),
                ("criterion", ctypes.c_int32), ("pre_out", ctypes.c_int32), ("post_out", ctypes.c_int32),
                ("min_corr", ctypes.c_float), ("max_corr", ctypes.c_float), ("ksize", ctypes.c_int32),
                ("semantics", ctypes.c_int32), ("rand_mode", ctypes.c_int32), ("precision", ctypes.c_int32)]


class RmtParams(ctypes.Structure):
    """kinc_rmt_params (include/kinc_rmt.h)."""
    _fields_ = [("threshold_start", ctypes.c_float), ("threshold_step", ctypes.c_float),
                ("threshold_stop", ctypes.c_float), ("chi_square_threshold1", ctypes.c_float),
                ("chi_square_threshold2", ctypes.c_float), ("min_eigenvalue_size", ctypes.c_int32),
                ("min_unfolding_pace", ctypes.c_int32), ("max_unfolding_pace", ctypes.c_int32),
                ("histogram_bin_size", ctypes.c_int32)]


RMT_ENOTHRESHOLD, RMT_ESPLINE = 6, 7


class Launch(ctypes.Structure):
    """kinc_sim_launch (include/kinc_sim.h): the per-pair kernel's launch shape."""
    _fields_ = [("warps_per_cta", ctypes.c_int32), ("rounds", ctypes.c_int32), ("prefetch", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]

    def as_dict(self):
        return {"warps_per_cta": self.warps_per_cta, "rounds": self.rounds, "prefetch": self.prefetch}


class TuneEntry(ctypes.Structure):
    """kinc_sim_tune_entry: one timed candidate of the autotuner."""
    _fields_ = [("launch", Launch), ("ms", ctypes.c_double)]

# name -> (restype, argtypes); every symbol include/kinc_sim.h declares
_VP = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
SIGNATURES = {
    "kinc_sim_tensor_peak": (ctypes.c_int, [_I32, ctypes.POINTER(ctypes.c_double)]),
    "kinc_sim_params_default": (ctypes.c_int, [ctypes.POINTER(SimParams)]),
    "kinc_sim_create": (ctypes.c_int, [_VP, _I32, _I32, ctypes.POINTER(SimParams), ctypes.POINTER(_VP)]),
    "kinc_sim_destroy": (None, [_VP]),
    "kinc_sim_last_error": (ctypes.c_char_p, [_VP]),
    "kinc_sim_total_pairs": (_I64, [_VP]),
    "kinc_sim_num_work_blocks": (_I32, [_VP]),
    "kinc_sim_execute_block": (ctypes.c_int, [_VP, _I64, _I64, _VP, _VP, _VP]),
    "kinc_sim_execute_block_async": (ctypes.c_int, [_VP, _I64, _I64, _VP, _VP, _VP]),
    "kinc_sim_execute_block_device": (ctypes.c_int, [_VP, _I64, _I64, _VP, _VP, _VP, _VP]),
    "kinc_sim_max_device_block": (_I64, [_VP]),
    "kinc_sim_synchronize": (ctypes.c_int, [_VP]),
    "kinc_sim_process_block": (ctypes.c_int, [_VP, _I64, _I64, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _I64,
                                              ctypes.POINTER(_I64), _VP, _VP, _VP, _VP, _I64,
                                              ctypes.POINTER(_I64)]),
    "kinc_sim_process_pairs": (ctypes.c_int, [ctypes.POINTER(SimParams), _I32, _I64, _I64, _VP, _VP, _VP, _VP,
                                              _VP, _VP, _VP, _I64, ctypes.POINTER(_I64), _VP, _VP, _VP, _VP,
                                              _I64, ctypes.POINTER(_I64)]),
    "kinc_sim_pair_counts": (ctypes.c_int, [_VP, _I64, _I64, _VP]),
    "kinc_sim_last_launch_count": (_I32, [_VP]),
    "kinc_sim_work_counters": (ctypes.c_int, [_VP, _VP, ctypes.c_int]),
    "kinc_sim_get_params": (ctypes.c_int, [_VP, ctypes.POINTER(SimParams), ctypes.POINTER(_I32),
                                           ctypes.POINTER(_I32)]),
    # include/kinc_pairwise_matrix.h
    "kinc_pm_create": (ctypes.c_int, [ctypes.c_char_p, _I32, _I32, _I32, _I32, _I32, ctypes.POINTER(_VP)]),
    "kinc_pm_write_items": (ctypes.c_int, [_VP, _I64, _VP, _VP, _VP, _VP]),
    "kinc_pm_close": (ctypes.c_int, [_VP]),
    "kinc_pm_write_items_packed": (ctypes.c_int, [_VP, _I64, _VP, _VP, _VP, _VP]),
    "kinc_sim_compact_block_device": (ctypes.c_int, [_VP, _I64, _I64, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _I64, _VP,
                                                     _VP, _VP, _VP, _I64, _VP, _VP]),
    "kinc_pm_open": (ctypes.c_int, [ctypes.c_char_p, _I32, _I32, ctypes.POINTER(_VP), ctypes.POINTER(_I32),
                                    ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(_I64),
                                    ctypes.POINTER(_I64)]),
    "kinc_pm_read_items": (ctypes.c_int, [_VP, _I64, _I64, _VP, _VP, _VP, _VP]),
    "kinc_emx_write": (ctypes.c_int, [ctypes.c_char_p, _VP, _I32, _I32, _I32]),
    "kinc_emx_read_header": (ctypes.c_int, [ctypes.c_char_p, _I32, ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "kinc_emx_read": (ctypes.c_int, [ctypes.c_char_p, _I32, _VP, _I64]),
    "kinc_pm_last_error": (ctypes.c_char_p, []),
    "kinc_sim_run_to_files": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_char_p, _I32, _I64, _I64]),
    "kinc_rmt_params_default": (None, [ctypes.POINTER(RmtParams)]),
    "kinc_rmt_run_items": (ctypes.c_int, [_I32, _I32, _I64, _VP, _VP, _VP, _VP, ctypes.POINTER(RmtParams),
                                           ctypes.c_char_p, ctypes.POINTER(ctypes.c_float), _VP, _I32,
                                           ctypes.POINTER(_I32)]),
    "kinc_rmt_run": (ctypes.c_int, [ctypes.c_char_p, _I32, ctypes.POINTER(RmtParams), ctypes.c_char_p,
                                     ctypes.POINTER(ctypes.c_float)]),
    "kinc_rmt_chi_square": (ctypes.c_int, [_VP, _I32, ctypes.POINTER(RmtParams), ctypes.POINTER(ctypes.c_float)]),
    "kinc_rmt_prune_eigenvalues": (ctypes.c_int, [_I32, _I32, _I64, _VP, _VP, _VP, _VP, ctypes.c_float, _VP,
                                                   ctypes.POINTER(_I32)]),
    "kinc_rmt_last_error": (ctypes.c_char_p, []),
    "kinc_pm_extract": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _I32,
                                        ctypes.c_float, ctypes.c_float, ctypes.c_char_p, ctypes.c_char_p]),
    "kinc_pm_export_text": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _I32, ctypes.c_char_p]),
    "kinc_shard_blocks": (ctypes.c_int, [_VP, _I32, _I32, ctypes.c_float, _I32, _I32, _I32,
                                         ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "kinc_pm_resume_point": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _I32, _I64,
                                            ctypes.POINTER(ctypes.c_int64)]),
    "kinc_pm_concat": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p), _I32, _I32]),
    "kinc_pm_import_text": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _I32, _I32, _I32, _I32]),
    "kinc_emx_import_text": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _I32, _I32, _I32, ctypes.c_char_p,
                                            ctypes.c_char_p, ctypes.c_char_p]),
    "kinc_emx_export_text": (ctypes.c_int, [ctypes.c_char_p, _I32, ctypes.c_char_p, ctypes.c_char_p, _I32,
                                            ctypes.c_char_p, ctypes.c_char_p]),
    "kinc_sim_run_to_files_ex": (ctypes.c_int, [_VP, ctypes.c_char_p, ctypes.c_char_p, _I32, _I64, _I64, _I64]),
    "kinc_sim_execute_block_noalloc": (ctypes.c_int, [_VP, _I32, _I32, ctypes.POINTER(SimParams), _I64, _I64,
                                                      _VP, _VP, _VP, _VP]),
    "kinc_sim_get_launch": (ctypes.c_int, [_VP, ctypes.POINTER(Launch)]),
    "kinc_sim_set_launch": (ctypes.c_int, [_VP, ctypes.POINTER(Launch)]),
    "kinc_sim_autotune": (ctypes.c_int, [_VP, _I64, _I64, _I32, ctypes.POINTER(Launch), ctypes.POINTER(TuneEntry),
                                         _I32, ctypes.POINTER(_I32)]),
}


def library_path():
    """The library to load: KINC_GB300_LIB overrides the in-tree build (A/B runs)."""
    return os.environ.get("KINC_GB300_LIB", _build.LIB)


def load(build_if_missing=True):
    """Load the native library, building it first if needed."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"native library {path} is missing; run kinc_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class SimError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"[{code}] {message}")
        self.code = code


def check(rc, ctx=None):
    if rc != OK:
        msg = load().kinc_sim_last_error(ctx)
        raise SimError(rc, msg.decode() if msg else "")
