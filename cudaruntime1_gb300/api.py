"""Python front end of libtsim.so.

Two layers, both calling the CUDA library through its C ABI:

* the reference's operator interface, same names and argument meaning as
  CudaRuntime1's headers (dtw.cuh, lcss.cuh, frechet.cuh, hausdorff.cuh,
  euclidean.cuh): host arrays in, one float per query out, plus the elapsed
  milliseconds the reference returns through ``float& gpu_time``;
* the exact kNN engine: a context, a device-resident candidate database and
  ``knn`` / ``knn_device`` returning top-k ids and distances;
* the serving loop (``Server``): continuous batching of requests of mixed
  measures and lengths, admitted by device-memory budget.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import (COST_EUCLID, COST_SQEUCLID, DTW, EUCLIDEAN, FLAG_ALWAYS_PRUNE,  # noqa: F401
                   FLAG_FP64_RESCORE, FLAG_NO_LANE_DP, FLAG_NO_WAVE_DP, FLAG_SHARE_THRESHOLDS,
                   FLAG_NO_GRAPH, FLAG_NO_PRUNE, FLAG_PLAIN, FRECHET, HAUSDORFF, LCSS,
                   TSIM_PENDING, TsimParams, TsimRequestInfo, TsimServerOpts, TsimServerStats,
                   TsimStats, check)

MEASURES = {"dtw": DTW, "lcss": LCSS, "frechet": FRECHET, "hausdorff": HAUSDORFF,
            "euclidean": EUCLIDEAN}


def _pts(a) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim == 1:
        a = a.reshape(-1, 2)
    if a.ndim != 2 or a.shape[1] != 2:
        raise ValueError(f"points must be [N, 2] float32, got shape {a.shape}")
    return a


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


# --------------------------------------------------------------- reference-named entry points
def _compat():
    return _lib.compat_symbols()


def _run_ref3(name, t1, t2, num_t, n, m, *extra):
    t1, t2 = _pts(t1), _pts(t2)
    if t1.shape[0] < num_t * n or t2.shape[0] < num_t * m:
        raise ValueError("trajectory arrays smaller than num_t * length")
    out = np.zeros(num_t, np.float32)
    gt = C.c_float(0.0)
    f = _compat()[name]
    f.restype = None
    args = [_ptr(t1), _ptr(t2), _ptr(out), C.c_int(num_t), C.c_int(n), C.c_int(m)]
    args += [C.c_float(e) for e in extra]
    args.append(C.byref(gt))
    f(*args)
    return out, gt.value


def launch_dtw_batch_gpu_knn(h_t1, h_t2, num_t, n, m):
    """CudaRuntime1/dtw.cuh:6 -- returns (h_results[num_t], gpu_time_ms)."""
    return _run_ref3("launch_dtw_batch_gpu_knn", h_t1, h_t2, num_t, n, m)


def launch_lcss_batch_gpu_wavefront_knn(h_t1, h_t2, num_t, n, m, epsilon):
    """CudaRuntime1/lcss.cuh:6-7 -- returns (h_results[num_t], gpu_time_ms)."""
    return _run_ref3("launch_lcss_batch_gpu_wavefront_knn", h_t1, h_t2, num_t, n, m, epsilon)


def launch_frechet_batch_gpu_wavefront(h_t1, h_t2, num_t, n, m):
    """CudaRuntime1/frechet.cuh:6 -- returns (h_results[num_t], gpu_time_ms)."""
    return _run_ref3("launch_frechet_batch_gpu_wavefront", h_t1, h_t2, num_t, n, m)


def run_hausdorff_rtree_gpu_pipeline(h_t1, num_t1, n, h_t2, num_t2, m, top_k=10):
    """CudaRuntime1/hausdorff.cuh:11-13 -- returns (h_results[num_t1], total_ms)."""
    t1, t2 = _pts(h_t1), _pts(h_t2)
    out = np.zeros(num_t1, np.float32)
    f = _compat()["run_hausdorff_rtree_gpu_pipeline"]
    f.restype = C.c_float
    ms = f(_ptr(t1), C.c_int(num_t1), C.c_int(n), _ptr(t2), C.c_int(num_t2), C.c_int(m), _ptr(out),
           C.c_int(top_k))
    return out, ms


def launch_hausdorff_rtree_gpu(h_t1, num_t1, n, h_t2, num_t2, m, h_candidate_indices, top_k):
    """CudaRuntime1/hausdorff.cuh:16-19 -- returns (h_results[num_t1], kernel_ms)."""
    t1, t2 = _pts(h_t1), _pts(h_t2)
    cand = np.ascontiguousarray(h_candidate_indices, np.int32)
    if cand.size < num_t1 * top_k:
        raise ValueError("candidate array smaller than num_t1 * top_k")
    out = np.zeros(num_t1, np.float32)
    gt = C.c_float(0.0)
    f = _compat()["launch_hausdorff_rtree_gpu"]
    f.restype = None
    f(_ptr(t1), C.c_int(num_t1), C.c_int(n), _ptr(t2), C.c_int(num_t2), C.c_int(m), _ptr(cand),
      C.c_int(top_k), _ptr(out), C.byref(gt))
    return out, gt.value


def launch_euclidean_batch_gpu_rtree_exact(h_t1, h_t2, num_t, n):
    """CudaRuntime1/euclidean.cuh:10 -- returns (h_results[num_t], total_ms)."""
    t1, t2 = _pts(h_t1), _pts(h_t2)
    out = np.zeros(num_t, np.float32)
    gt = C.c_float(0.0)
    f = _compat()["launch_euclidean_batch_gpu_rtree_exact"]
    f.restype = None
    f(_ptr(t1), _ptr(t2), _ptr(out), C.c_int(num_t), C.c_int(n), C.byref(gt))
    return out, gt.value


def execute_rtree_csr_kernel_on_gpu(h_t1, h_t2, h_candidates, h_offsets, num_t, n,
                                    total_candidates):
    """CudaRuntime1/euclidean.cuh:11-13 -- returns (h_results[num_t], kernel_ms)."""
    t1, t2 = _pts(h_t1), _pts(h_t2)
    cand = np.ascontiguousarray(h_candidates, np.int32)
    off = np.ascontiguousarray(h_offsets, np.int32)
    out = np.zeros(num_t, np.float32)
    gt = C.c_float(0.0)
    f = _compat()["execute_rtree_csr_kernel_on_gpu"]
    f.restype = None
    f(_ptr(t1), _ptr(t2), _ptr(cand), _ptr(off), _ptr(out), C.c_int(num_t), C.c_int(n),
      C.c_int(total_candidates), C.byref(gt))
    return out, gt.value


# --------------------------------------------------------------- engine
class Context:
    """A tsim context: CUDA device, stream and scratch arena."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self.L = _lib.load()
        h = C.c_void_p()
        check(self.L.tsim_ctx_create(device, C.c_void_p(stream or 0), C.byref(h)))
        self.h = h
        self.device = device

    def set_stream(self, stream: int | None):
        check(self.L.tsim_ctx_set_stream(self.h, C.c_void_p(stream or 0)))

    def synchronize(self):
        check(self.L.tsim_ctx_synchronize(self.h))

    def scratch_bytes(self) -> int:
        return self.L.tsim_ctx_scratch_bytes(self.h)

    def set_profiling(self, on: bool):
        """Per-stage CUDA-event timing on the context stream."""
        check(self.L.tsim_ctx_set_profiling(self.h, 1 if on else 0))

    def counters(self, reset: bool = True) -> dict:
        """Stage times (ms), stage calls, kernels launched, DP cells computed
        since the last reset (synchronises the stream)."""
        n = len(_lib.STAGES)
        ms = (C.c_double * n)()
        calls = (C.c_int64 * n)()
        launches, cells = C.c_int64(), C.c_int64()
        check(self.L.tsim_ctx_counters(self.h, ms, calls, C.byref(launches), C.byref(cells),
                                       1 if reset else 0))
        return {"stage_ms": {s: ms[i] for i, s in enumerate(_lib.STAGES)},
                "stage_calls": {s: calls[i] for i, s in enumerate(_lib.STAGES)},
                "launches": launches.value, "dp_cells": cells.value}

    def set_concurrency(self, streams: int):
        """Streams one kNN request may use (chunks of queries overlap)."""
        check(self.L.tsim_ctx_set_concurrency(self.h, streams))

    def autotune(self, db, qpts_ptr: int, qoff_ptr: int, nq: int, max_qlen: int, measure: str,
                 k: int = 10, reps: int = 5, **kw) -> dict:
        """Time the launch choices on this request (device pointers) and keep
        the fastest for its shape class (tsim_autotune)."""
        p = make_params(measure, k, **kw)
        r = _lib.TsimTuneResult()
        check(self.L.tsim_autotune(self.h, C.byref(p), C.c_void_p(qpts_ptr), C.c_void_p(qoff_ptr),
                                   nq, max_qlen, db.h, reps, C.byref(r)))
        return r.as_dict()

    def save_tuning(self, path: str):
        check(self.L.tsim_tuning_save(self.h, str(path).encode()))

    def load_tuning(self, path: str):
        check(self.L.tsim_tuning_load(self.h, str(path).encode()))

    def clear_tuning(self):
        check(self.L.tsim_tuning_clear(self.h))

    def tuning_count(self) -> int:
        return self.L.tsim_tuning_count(self.h)

    def survivor_cells(self) -> int:
        """DP cells of the survivor round since the last counter reset."""
        v = C.c_int64()
        check(self.L.tsim_ctx_survivor_cells(self.h, C.byref(v)))
        return v.value

    def probe_fp32_tflops(self) -> float:
        v = C.c_double()
        check(self.L.tsim_probe_fp32_tflops(self.h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "h", None):
            self.L.tsim_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Database:
    """Device-resident candidate set (CSR trajectories + summaries)."""

    def __init__(self, ctx: Context, pts=None, off=None, *, device_pts=None, device_off=None,
                 count=None, max_len=0, path=None):
        self.ctx = ctx
        self.L = ctx.L
        h = C.c_void_p()
        if path is not None:  # a file written by save()
            check(self.L.tsim_db_load(ctx.h, str(path).encode(), C.byref(h)))
            self._keep = None
        elif device_pts is not None:
            check(self.L.tsim_db_wrap_device(ctx.h, C.c_void_p(device_pts),
                                             C.c_void_p(device_off), count, max_len, C.byref(h)))
            self._keep = None
        else:
            pts = _pts(pts)
            off = np.ascontiguousarray(off, np.int64)
            self._keep = (pts, off)
            check(self.L.tsim_db_create(ctx.h, _ptr(pts), _ptr(off), len(off) - 1, C.byref(h)))
        self.h = h

    @property
    def count(self) -> int:
        return self.L.tsim_db_count(self.h)

    def device_bytes(self) -> int:
        return self.L.tsim_db_device_bytes(self.h)

    def save(self, path):
        check(self.L.tsim_db_save(self.h, str(path).encode()))

    def close(self):
        if getattr(self, "h", None):
            self.L.tsim_db_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_params(measure: str, k: int = 10, *, cost: int = COST_SQEUCLID, band_pct: int = -1,
                epsilon: float = 0.5, delta: int = -1, flags: int = 0) -> TsimParams:
    return TsimParams(MEASURES[measure], k, cost, band_pct, epsilon, delta, flags)


def knn(ctx: Context, db: Database, qpts, qoff, measure: str, k: int = 10, stats: bool = True,
        **kw):
    """Exact kNN with host arrays end to end.  Returns (ids[nq,k], dists[nq,k],
    stats dict or None).  Without stats, repeated requests of one shape replay a
    captured CUDA graph."""
    qpts = _pts(qpts)
    qoff = np.ascontiguousarray(qoff, np.int64)
    nq = len(qoff) - 1
    ids = np.zeros(nq * k, np.int32)
    d = np.zeros(nq * k, np.float32)
    st = TsimStats() if stats else None
    p = make_params(measure, k, **kw)
    check(ctx.L.tsim_knn_host(ctx.h, C.byref(p), _ptr(qpts), _ptr(qoff), nq, db.h, _ptr(ids),
                              _ptr(d), C.byref(st) if st is not None else None))
    return ids.reshape(nq, k), d.reshape(nq, k), (st.as_dict() if st is not None else None)


def knn_device(ctx: Context, db: Database, qpts_ptr: int, qoff_ptr: int, nq: int, max_qlen: int,
               ids_ptr: int, dists_ptr: int, dists64_ptr: int | None, measure: str, k: int = 10,
               stats: bool = False, **kw):
    """Exact kNN on device pointers (e.g. torch tensors' data_ptr()).  Runs
    asynchronously on the context stream unless ``stats`` is set."""
    p = make_params(measure, k, **kw)
    st = TsimStats() if stats else None
    check(ctx.L.tsim_knn(ctx.h, C.byref(p), C.c_void_p(qpts_ptr), C.c_void_p(qoff_ptr), nq,
                         max_qlen, db.h, C.c_void_p(ids_ptr), C.c_void_p(dists_ptr),
                         C.c_void_p(dists64_ptr or 0), C.byref(st) if st is not None else None))
    return st.as_dict() if st is not None else None


def ref_batch_device(ctx: Context, measure: str, t1_ptr: int, t2_ptr: int, num_t: int, n: int,
                     m: int, out_ptr: int, epsilon: float = 0.5):
    check(ctx.L.tsim_ref_batch(ctx.h, MEASURES[measure], C.c_void_p(t1_ptr), C.c_void_p(t2_ptr),
                               num_t, n, m, C.c_float(epsilon), C.c_void_p(out_ptr)))


def band_cells(ctx: Context, db: Database, qpts_ptr: int, qoff_ptr: int, nq: int, measure: str,
               **kw) -> int:
    """Band cells of every query x database pair (the unpruned DP work)."""
    p = make_params(measure, 1, **kw)
    v = C.c_int64()
    check(ctx.L.tsim_band_cells(ctx.h, C.byref(p), C.c_void_p(qpts_ptr), C.c_void_p(qoff_ptr), nq,
                                db.h, C.byref(v)))
    return v.value


def dp_pairs(ctx: Context, measure: str, precision: int, kernel: int, qpts_ptr: int, qoff_ptr: int,
             max_qlen: int, cpts_ptr: int, coff_ptr: int, max_clen: int, pairs_ptr: int,
             npairs: int, out32_ptr: int = 0, out64_ptr: int = 0, **kw):
    """DP values of explicit (query, candidate) pairs on the device
    (tsim_dp_pairs): precision 0 FP32, 1 compensated, 2 FP64; kernel 0 auto,
    1 round-striped, 2 anti-diagonal."""
    p = make_params(measure, 1, **kw)
    check(ctx.L.tsim_dp_pairs(ctx.h, C.byref(p), precision, kernel, C.c_void_p(qpts_ptr),
                              C.c_void_p(qoff_ptr), max_qlen, C.c_void_p(cpts_ptr),
                              C.c_void_p(coff_ptr), max_clen, C.c_void_p(pairs_ptr), npairs,
                              C.c_void_p(out32_ptr), C.c_void_p(out64_ptr)))


class Server:
    """Continuous-batching request loop over a resident database
    (tsim_server_*): ``submit`` returns a ticket at once; the library's worker
    thread admits requests into free stream slots while their scratch fits
    the device pool, so requests of any measure and length overlap on the GPU."""

    def __init__(self, ctx: Context, db: Database, slots: int = 16,
                 hbm_budget_bytes: int = 1 << 30, queue_cap: int = 65536):
        self.ctx, self.db, self.L = ctx, db, ctx.L
        opts = TsimServerOpts(slots, hbm_budget_bytes, queue_cap)
        h = C.c_void_p()
        check(self.L.tsim_server_create(ctx.h, db.h, C.byref(opts), C.byref(h)))
        self.h = h
        self._k = {}

    def submit(self, qpts, qoff, measure: str, k: int = 10, **kw) -> int:
        qpts = _pts(qpts)
        qoff = np.ascontiguousarray(qoff, np.int64)
        p = make_params(measure, k, **kw)
        t = C.c_uint64()
        check(self.L.tsim_server_submit(self.h, C.byref(p), _ptr(qpts), _ptr(qoff), len(qoff) - 1,
                                        C.byref(t)))
        self._k[t.value] = (len(qoff) - 1, k)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        """(ids[nq,k], dists[nq,k], info dict); None if still pending."""
        nq, k = self._k[ticket]
        ids = np.zeros(nq * k, np.int32)
        d = np.zeros(nq * k, np.float32)
        info = TsimRequestInfo()
        st = self.L.tsim_server_wait(self.h, ticket, timeout_ms, _ptr(ids), _ptr(d),
                                     C.byref(info))
        if st == TSIM_PENDING:
            return None
        del self._k[ticket]
        check(st)
        return ids.reshape(nq, k), d.reshape(nq, k), info.as_dict()

    def stats(self) -> dict:
        st = TsimServerStats()
        check(self.L.tsim_server_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    def close(self):
        if getattr(self, "h", None):
            self.L.tsim_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def knn_scratch_bytes(db: Database, measure: str, nq: int, max_qlen: int, k: int = 10,
                      **kw) -> int:
    p = make_params(measure, k, **kw)
    return int(db.L.tsim_knn_scratch_bytes(C.byref(p), nq, max_qlen, db.h))
