"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker or as the timed CPU
baseline.  The product library never loads it.

``liboracle.so`` is the C restatement in oracle.c (built by ``make`` in this
directory).  ``_ref/libref.so`` is the reference's own CPU code
(CudaRuntime1/dtw.cpp, lcss.cpp, frechet.cpp) compiled in place by
``make ref``; it only exists where the reference checkout is present.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None
_LOCK = threading.Lock()

DTW, LCSS, FRECHET, HAUSDORFF, EUCLIDEAN = range(5)
COST_SQEUCLID, COST_EUCLID = 0, 1
MEASURES = {"dtw": DTW, "lcss": LCSS, "frechet": FRECHET, "hausdorff": HAUSDORFF,
            "euclidean": EUCLIDEAN}

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int)
_i64p = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)


class OrcParams(C.Structure):
    _fields_ = [("measure", C.c_int), ("k", C.c_int), ("cost", C.c_int),
                ("band_pct", C.c_int), ("epsilon", C.c_float), ("delta", C.c_int)]


# where the reference's sources are read from: TSIM_REFERENCE_DIR, else a
# checkout named reference/ beside this repository (absent on most machines)
REFERENCE_DIR_DEFAULT = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference",
                                     "CudaRuntime1")


def reference_dir():
    """The directory holding the reference's dtw.cpp, lcss.cpp, frechet.cpp,
    or None where there is none."""
    d = os.environ.get("TSIM_REFERENCE_DIR") or REFERENCE_DIR_DEFAULT
    return d if os.path.isfile(os.path.join(d, "dtw.cpp")) else None


def build(ref: bool = True) -> None:
    """Compile liboracle.so (always) and _ref/libref.so (when the reference
    sources are present), passing the reference directory to make."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    d = reference_dir()
    if ref and d:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "refgpu", "REF=" + os.path.abspath(d)],
                       check=True)


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = os.path.join(HERE, "liboracle.so")
            if not os.path.exists(path):
                subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
            L = C.CDLL(path)
            L.orc_ref_dtw.argtypes = [_fp, _fp, _fp, C.c_int, C.c_int, C.c_int]
            L.orc_ref_dtw.restype = C.c_float
            L.orc_ref_frechet.argtypes = [_fp, _fp, _fp, C.c_int, C.c_int, C.c_int]
            L.orc_ref_frechet.restype = C.c_float
            L.orc_ref_lcss.argtypes = [_fp, _fp, _fp, C.c_int, C.c_int, C.c_int, C.c_float]
            L.orc_ref_lcss.restype = C.c_float
            L.orc_ref_directed_hausdorff_grid.argtypes = [_fp, C.c_int, _fp, C.c_int, C.c_float]
            L.orc_ref_directed_hausdorff_grid.restype = C.c_float
            L.orc_ref_hausdorff_cands.argtypes = [_fp, C.c_int, C.c_int, _fp, C.c_int, C.c_int,
                                                  _ip, C.c_int, _fp]
            L.orc_ref_euclid_cands.argtypes = [_fp, _fp, _ip, _ip, _fp, C.c_int, C.c_int]
            L.orc_mbr_knn.argtypes = [_fp, C.c_int, C.c_int, _fp, C.c_int, C.c_int, C.c_int, _ip]
            L.orc_dtw64.argtypes = [_fp, C.c_int, _fp, C.c_int, C.c_int, C.c_int]
            L.orc_dtw64.restype = C.c_double
            L.orc_lcss_count.argtypes = [_fp, C.c_int, _fp, C.c_int, C.c_float, C.c_int]
            L.orc_lcss_count.restype = C.c_int
            for f in ("orc_frechet64", "orc_hausdorff64"):
                getattr(L, f).argtypes = [_fp, C.c_int, _fp, C.c_int]
                getattr(L, f).restype = C.c_double
            L.orc_euclid64.argtypes = [_fp, C.c_int, _fp, C.c_int]
            L.orc_euclid64.restype = C.c_double
            L.orc_band_w.argtypes = [C.c_int, C.c_int, C.c_int]
            L.orc_band_w.restype = C.c_int
            L.orc_band_row.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _ip, _ip]
            L.orc_knn.argtypes = [C.POINTER(OrcParams), _fp, _i64p, C.c_int, _fp, _i64p, C.c_int,
                                  _ip, _dp, C.c_int]
            L.orc_dtw_knn_pruned.argtypes = [C.POINTER(OrcParams), _fp, _i64p, C.c_int, _fp,
                                             _i64p, C.c_int, _ip, _dp, C.c_int, _i64p]
            L.orc_knn_pruned.argtypes = [C.POINTER(OrcParams), _fp, _i64p, C.c_int, _fp, _i64p,
                                         C.c_int, _ip, _dp, C.c_int, _i64p]
            L.orc_num_threads.restype = C.c_int
            _LIB = L
    return _LIB


def ref_lib():
    """The reference's own CPU functions, or None when they were not built."""
    global _REF
    with _LOCK:
        if _REF is None:
            path = os.path.join(HERE, "_ref", "libref.so")
            if not os.path.exists(path):
                return None
            L = C.CDLL(path)
            for f in ("ref_dtw_cpu", "ref_frechet_cpu"):
                getattr(L, f).argtypes = [_fp, _fp, _fp, C.c_int, C.c_int, C.c_int]
                getattr(L, f).restype = C.c_float
            L.ref_lcss_cpu.argtypes = [_fp, _fp, _fp, C.c_int, C.c_int, C.c_int, C.c_float]
            L.ref_lcss_cpu.restype = C.c_float
            _REF = L
    return _REF


def _f(a):
    return a.ctypes.data_as(_fp)


def _pts(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a


# ---------------------------------------------------------------- reference semantics
def ref_batch(measure: str, t1, t2, n: int, m: int, eps: float = 0.5, use_ref: bool = False):
    """One float per query, the reference's batch semantics.  ``use_ref``
    runs the reference's own compiled CPU code instead of the restatement."""
    t1 = _pts(t1)
    t2 = _pts(t2)
    num_t = t1.size // (2 * n)
    out = np.zeros(num_t, np.float32)
    if use_ref:
        L = ref_lib()
        if L is None:
            raise RuntimeError("oracle/_ref/libref.so not built")
        fn = {"dtw": L.ref_dtw_cpu, "lcss": L.ref_lcss_cpu, "frechet": L.ref_frechet_cpu}[measure]
    else:
        L = lib()
        fn = {"dtw": L.orc_ref_dtw, "lcss": L.orc_ref_lcss, "frechet": L.orc_ref_frechet}[measure]
    if measure == "lcss":
        fn(_f(t1), _f(t2), _f(out), num_t, n, m, C.c_float(eps))
    else:
        fn(_f(t1), _f(t2), _f(out), num_t, n, m)
    return out


def ref_hausdorff_cands(t1, n, t2, m, cand):
    t1, t2 = _pts(t1), _pts(t2)
    cand = np.ascontiguousarray(cand, np.int32)
    num_t1 = t1.size // (2 * n)
    top_k = cand.size // num_t1
    out = np.zeros(num_t1, np.float32)
    lib().orc_ref_hausdorff_cands(_f(t1), num_t1, n, _f(t2), t2.size // (2 * m), m,
                                  cand.ctypes.data_as(_ip), top_k, _f(out))
    return out


def ref_euclid_cands(t1, t2, n, cand, offsets):
    t1, t2 = _pts(t1), _pts(t2)
    cand = np.ascontiguousarray(cand, np.int32)
    offsets = np.ascontiguousarray(offsets, np.int32)
    num_t = t1.size // (2 * n)
    out = np.zeros(num_t, np.float32)
    lib().orc_ref_euclid_cands(_f(t1), _f(t2), cand.ctypes.data_as(_ip),
                               offsets.ctypes.data_as(_ip), _f(out), num_t, n)
    return out


def mbr_knn(t1, n, t2, m, k):
    t1, t2 = _pts(t1), _pts(t2)
    num_t1 = t1.size // (2 * n)
    out = np.zeros(num_t1 * k, np.int32)
    lib().orc_mbr_knn(_f(t1), num_t1, n, _f(t2), t2.size // (2 * m), m, k,
                      out.ctypes.data_as(_ip))
    return out


def directed_hausdorff_grid(src, tgt, seed=0.0):
    src, tgt = _pts(src), _pts(tgt)
    return lib().orc_ref_directed_hausdorff_grid(_f(src), src.size // 2, _f(tgt), tgt.size // 2,
                                                 C.c_float(seed))


# ---------------------------------------------------------------- FP64 exact
def band_w(n, m, band_pct):
    return lib().orc_band_w(n, m, band_pct)


def band_row(i, n, m, w):
    lo, hi = C.c_int(), C.c_int()
    lib().orc_band_row(i, n, m, w, C.byref(lo), C.byref(hi))
    return lo.value, hi.value


def pair(measure: str, a, b, *, band_pct=-1, cost=COST_SQEUCLID, eps=0.5, delta=-1):
    a, b = _pts(a), _pts(b)
    n, m = a.size // 2, b.size // 2
    L = lib()
    if measure == "dtw":
        return L.orc_dtw64(_f(a), n, _f(b), m, band_pct, cost)
    if measure == "lcss":
        return L.orc_lcss_count(_f(a), n, _f(b), m, C.c_float(eps), delta)
    if measure == "frechet":
        return L.orc_frechet64(_f(a), n, _f(b), m)
    if measure == "hausdorff":
        return L.orc_hausdorff64(_f(a), n, _f(b), m)
    return L.orc_euclid64(_f(a), n, _f(b), m)


def _params(measure, k, cost, band_pct, eps, delta):
    return OrcParams(MEASURES[measure], k, cost, band_pct, eps, delta)


def knn(measure: str, qpts, qoff, dbpts, dboff, k: int, *, band_pct=-1, cost=COST_SQEUCLID,
        eps=0.5, delta=-1, nthreads=0):
    """Brute-force exact kNN over CSR trajectory sets.  Returns (ids, dists)
    shaped [nq, k]; for LCSS ``dists`` holds the integer match counts."""
    qpts, dbpts = _pts(qpts), _pts(dbpts)
    qoff = np.ascontiguousarray(qoff, np.int64)
    dboff = np.ascontiguousarray(dboff, np.int64)
    nq, ndb = len(qoff) - 1, len(dboff) - 1
    ids = np.zeros(nq * k, np.int32)
    d = np.zeros(nq * k, np.float64)
    p = _params(measure, k, cost, band_pct, eps, delta)
    lib().orc_knn(C.byref(p), _f(qpts), qoff.ctypes.data_as(_i64p), nq, _f(dbpts),
                  dboff.ctypes.data_as(_i64p), ndb, ids.ctypes.data_as(_ip),
                  d.ctypes.data_as(_dp), nthreads)
    return ids.reshape(nq, k), d.reshape(nq, k)


def dtw_knn_pruned(qpts, qoff, dbpts, dboff, k: int, *, band_pct=-1, cost=COST_SQEUCLID,
                   nthreads=0):
    """Exact DTW kNN with lower-bound pruning (the CPU baseline).  Returns
    (ids, dists, dp_cells)."""
    qpts, dbpts = _pts(qpts), _pts(dbpts)
    qoff = np.ascontiguousarray(qoff, np.int64)
    dboff = np.ascontiguousarray(dboff, np.int64)
    nq, ndb = len(qoff) - 1, len(dboff) - 1
    ids = np.zeros(nq * k, np.int32)
    d = np.zeros(nq * k, np.float64)
    cells = C.c_int64(0)
    p = _params("dtw", k, cost, band_pct, 0.0, -1)
    lib().orc_dtw_knn_pruned(C.byref(p), _f(qpts), qoff.ctypes.data_as(_i64p), nq, _f(dbpts),
                             dboff.ctypes.data_as(_i64p), ndb, ids.ctypes.data_as(_ip),
                             d.ctypes.data_as(_dp), nthreads, C.byref(cells))
    return ids.reshape(nq, k), d.reshape(nq, k), cells.value


def knn_pruned(measure: str, qpts, qoff, dbpts, dboff, k: int, *, band_pct=-1,
               cost=COST_SQEUCLID, eps=0.5, delta=-1, nthreads=0, evaluated=False):
    """Exact kNN with FP64 bound pruning (same results as ``knn``, ties
    included), for parity checks against large databases.  Returns (ids,
    dists) or, with ``evaluated``, (ids, dists, candidates evaluated)."""
    qpts, dbpts = _pts(qpts), _pts(dbpts)
    qoff = np.ascontiguousarray(qoff, np.int64)
    dboff = np.ascontiguousarray(dboff, np.int64)
    nq, ndb = len(qoff) - 1, len(dboff) - 1
    ids = np.zeros(nq * k, np.int32)
    d = np.zeros(nq * k, np.float64)
    ev = C.c_int64(0)
    p = _params(measure, k, cost, band_pct, eps, delta)
    lib().orc_knn_pruned(C.byref(p), _f(qpts), qoff.ctypes.data_as(_i64p), nq, _f(dbpts),
                         dboff.ctypes.data_as(_i64p), ndb, ids.ctypes.data_as(_ip),
                         d.ctypes.data_as(_dp), nthreads, C.byref(ev))
    out = (ids.reshape(nq, k), d.reshape(nq, k))
    return out + (ev.value,) if evaluated else out


def num_threads() -> int:
    return lib().orc_num_threads()
