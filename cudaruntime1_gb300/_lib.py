"""ctypes bindings of libtsim.so (include/tsim.h and include/compat/*.cuh).

The library is the product: every function here calls into CUDA code.  If
the library has not been built, loading raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import buildlib as _build

_LIB = None
_LOCK = threading.Lock()

TSIM_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
          4: "timeout", 5: "unsupported", 6: "over budget", 7: "pending", 8: "queue full"}
TSIM_ERR_INVALID_ARG = 1
TSIM_ERR_BUDGET, TSIM_PENDING, TSIM_ERR_BUSY = 6, 7, 8

DTW, LCSS, FRECHET, HAUSDORFF, EUCLIDEAN = range(5)
COST_SQEUCLID, COST_EUCLID = 0, 1
FLAG_NO_PRUNE, FLAG_PLAIN, FLAG_NO_GRAPH, FLAG_FP64_RESCORE, FLAG_ALWAYS_PRUNE = 1, 2, 4, 8, 16
FLAG_NO_LANE_DP, FLAG_NO_WAVE_DP, FLAG_SHARE_THRESHOLDS = 32, 64, 128
STAGES = ["summary", "lb1", "seed", "filter", "dp", "select", "rescore", "ref", "dp_survivors"]

_vp = C.c_void_p
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


class TsimParams(C.Structure):
    _fields_ = [("measure", C.c_int), ("k", C.c_int), ("cost", C.c_int), ("band_pct", C.c_int),
                ("epsilon", C.c_float), ("delta", C.c_int), ("flags", C.c_uint)]


class TsimStats(C.Structure):
    _fields_ = [("ms", C.c_double), ("pairs", C.c_int64), ("pairs_lb1", C.c_int64),
                ("pairs_lb2", C.c_int64), ("pairs_refined", C.c_int64),
                ("cells", C.c_int64), ("cells_unpruned", C.c_int64), ("rescored", C.c_int64),
                ("rescored_fp64", C.c_int64),
                ("launches", C.c_int32), ("graph_replay", C.c_int32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class TsimServerOpts(C.Structure):
    _fields_ = [("slots", C.c_int), ("hbm_budget_bytes", C.c_int64), ("queue_cap", C.c_int)]


class TsimRequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("nq", C.c_int), ("k", C.c_int), ("queue_ms", C.c_double),
                ("latency_ms", C.c_double), ("device_ms", C.c_double),
                ("scratch_bytes", C.c_int64), ("inflight_at_admit", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class TsimServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("rejected", C.c_int64), ("queued", C.c_int), ("in_flight", C.c_int),
                ("peak_in_flight", C.c_int), ("slots", C.c_int), ("budget_bytes", C.c_int64),
                ("scratch_in_use", C.c_int64), ("peak_scratch_bytes", C.c_int64),
                ("launch_ms", C.c_double), ("busy_ms", C.c_double),
                ("shared_threshold_hits", C.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class TsimTuneResult(C.Structure):
    _fields_ = [("rdiag", C.c_int), ("streams", C.c_int), ("best_ms", C.c_double),
                ("default_ms", C.c_double), ("tried", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class TsimError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"tsim: {STATUS.get(status, status)}: {msg}")
        self.status = status


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libtsim.so.  Raises if it is missing (or builds it when asked)."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = os.environ.get("TSIM_LIB") or _build.LIB  # e.g. the bounds-checked build
        if path != _build.LIB:
            if not os.path.exists(path):
                raise RuntimeError(f"TSIM_LIB={path} does not exist")
        elif not os.path.exists(_build.LIB):
            if not build_if_missing:
                raise RuntimeError(
                    f"{_build.LIB} is not built: run cudaruntime1_gb300.build() "
                    "(nvcc, sm_103a); there is no CPU fallback")
            _build.build()
        L = C.CDLL(path)
        sig = {
            "tsim_status_string": ([C.c_int], C.c_char_p),
            "tsim_last_error": ([], C.c_char_p),
            "tsim_version": ([], C.c_int),
            "tsim_ctx_create": ([C.c_int, _vp, C.POINTER(_vp)], C.c_int),
            "tsim_ctx_destroy": ([_vp], C.c_int),
            "tsim_ctx_set_stream": ([_vp, _vp], C.c_int),
            "tsim_ctx_synchronize": ([_vp], C.c_int),
            "tsim_ctx_scratch_bytes": ([_vp], C.c_int64),
            "tsim_db_create": ([_vp, _vp, _vp, C.c_int, C.POINTER(_vp)], C.c_int),
            "tsim_db_wrap_device": ([_vp, _vp, _vp, C.c_int, C.c_int, C.POINTER(_vp)], C.c_int),
            "tsim_db_destroy": ([_vp], C.c_int),
            "tsim_db_save": ([_vp, C.c_char_p], C.c_int),
            "tsim_db_load": ([_vp, C.c_char_p, C.POINTER(_vp)], C.c_int),
            "tsim_db_count": ([_vp], C.c_int),
            "tsim_db_device_bytes": ([_vp], C.c_int64),
            "tsim_knn": ([_vp, C.POINTER(TsimParams), _vp, _vp, C.c_int, C.c_int, _vp, _vp, _vp,
                          _vp, C.POINTER(TsimStats)], C.c_int),
            "tsim_knn_host": ([_vp, C.POINTER(TsimParams), _vp, _vp, C.c_int, _vp, _vp, _vp,
                               C.POINTER(TsimStats)], C.c_int),
            "tsim_ref_batch": ([_vp, C.c_int, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_float, _vp],
                               C.c_int),
            "tsim_hausdorff_cands": ([_vp, _vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, _vp,
                                      C.c_int, _vp], C.c_int),
            "tsim_euclid_cands": ([_vp, _vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp],
                                  C.c_int),
            "tsim_mbr_knn": ([_vp, _vp, C.c_int, C.c_int, _vp, C.c_int, C.c_int, C.c_int, _vp],
                             C.c_int),
            "tsim_ctx_set_profiling": ([_vp, C.c_int], C.c_int),
            "tsim_ctx_counters": ([_vp, C.POINTER(C.c_double), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int], C.c_int),
            "tsim_probe_fp32_tflops": ([_vp, C.POINTER(C.c_double)], C.c_int),
            "tsim_debug_fail_allocations": ([C.c_int, C.c_int], C.c_int),
            "tsim_debug_set_canary": ([C.c_int], C.c_int),
            "tsim_debug_set_wait_limit": ([C.c_int64], C.c_int),
            "tsim_debug_bounds_violations": ([C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
                                             C.c_int),
            "tsim_ctx_set_concurrency": ([_vp, C.c_int], C.c_int),
            "tsim_ctx_survivor_cells": ([_vp, C.POINTER(C.c_int64)], C.c_int),
            "tsim_band_cells": ([_vp, C.POINTER(TsimParams), _vp, _vp, C.c_int, _vp,
                                 C.POINTER(C.c_int64)], C.c_int),
            "tsim_autotune": ([_vp, C.POINTER(TsimParams), _vp, _vp, C.c_int, C.c_int, _vp, C.c_int,
                               C.POINTER(TsimTuneResult)], C.c_int),
            "tsim_tuning_save": ([_vp, C.c_char_p], C.c_int),
            "tsim_tuning_load": ([_vp, C.c_char_p], C.c_int),
            "tsim_tuning_clear": ([_vp], C.c_int),
            "tsim_tuning_count": ([_vp], C.c_int),
            "tsim_knn_scratch_bytes": ([C.POINTER(TsimParams), C.c_int, C.c_int, _vp], C.c_int64),
            "tsim_server_create": ([_vp, _vp, C.POINTER(TsimServerOpts), C.POINTER(_vp)], C.c_int),
            "tsim_server_submit": ([_vp, C.POINTER(TsimParams), _vp, _vp, C.c_int,
                                    C.POINTER(C.c_uint64)], C.c_int),
            "tsim_server_wait": ([_vp, C.c_uint64, C.c_int, _vp, _vp, C.POINTER(TsimRequestInfo)],
                                 C.c_int),
            "tsim_server_get_stats": ([_vp, C.POINTER(TsimServerStats)], C.c_int),
            "tsim_server_destroy": ([_vp], C.c_int),
            "tsim_dp_pairs": ([_vp, C.POINTER(TsimParams), C.c_int, C.c_int, _vp, _vp, C.c_int,
                               _vp, _vp, C.c_int, _vp, C.c_int, _vp, _vp], C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _LIB = L
        return L


def check(status: int):
    if status != TSIM_OK:
        raise TsimError(status, load().tsim_last_error().decode(errors="replace"))


# the reference-named C++ entry points (C++ linkage): their Itanium-ABI names
# for the reference's exact signatures (tests/test_abi.py demangles and checks them)
def compat_symbols():
    """Map reference function name -> ctypes function of libtsim.so."""
    L = load()
    names = {
        "launch_dtw_batch_gpu_knn": "_Z24launch_dtw_batch_gpu_knnPK5PointS1_PfiiiRf",
        "launch_lcss_batch_gpu_wavefront_knn":
            "_Z35launch_lcss_batch_gpu_wavefront_knnPK5PointS1_PfiiifRf",
        "launch_frechet_batch_gpu_wavefront":
            "_Z34launch_frechet_batch_gpu_wavefrontPK5PointS1_PfiiiRf",
        "run_hausdorff_rtree_gpu_pipeline":
            "_Z32run_hausdorff_rtree_gpu_pipelinePK5PointiiS1_iiPfi",
        "launch_hausdorff_rtree_gpu": "_Z26launch_hausdorff_rtree_gpuPK5PointiiS1_iiPKiiPfRf",
        "launch_euclidean_batch_gpu_rtree_exact":
            "_Z38launch_euclidean_batch_gpu_rtree_exactPK5PointS1_PfiiRf",
        "execute_rtree_csr_kernel_on_gpu": "_Z31execute_rtree_csr_kernel_on_gpuPK5PointS1_PKiS3_PfiiiRf",
    }
    out = {}
    for ref, mangled in names.items():
        out[ref] = getattr(L, mangled)
    return out
