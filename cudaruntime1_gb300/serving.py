"""Load generator for the serving loop (``Server``): a device-resident
database of random-walk trajectories, kNN requests of mixed measures and
query lengths arriving as a Poisson process, latency percentiles and
achieved throughput.

Per-measure parameters follow the batched workloads: DTW with a 10 % band
and squared cost, LCSS with epsilon 0.25 and index window 20, discrete
Frechet, symmetric Hausdorff, lock-step Euclidean.
"""
from __future__ import annotations

import threading
import time

import numpy as np

from . import api
from . import datagen as G

MEASURE_PARAMS = {
    "dtw": dict(band_pct=10, cost=api.COST_SQEUCLID),
    "lcss": dict(epsilon=0.25, delta=20),
    "frechet": dict(),
    "hausdorff": dict(),
    "euclidean": dict(),
}


def device_random_walks(count: int, lo: int, hi: int, seed: int, device="cuda",
                        keep_host: bool = False):
    """``count`` random walks with lengths U[lo, hi] (start uniform in
    [0,100]^2, N(0,1) steps per coordinate), generated on the host with
    numpy's seeded generator and copied to ``device``.  Returns (points
    float32 [total, 2], offsets int64 [count+1], max_len) as torch tensors,
    followed by the host arrays (points, offsets) when ``keep_host``."""
    import torch
    rng = np.random.default_rng(seed)
    lens = rng.integers(lo, hi + 1, count).astype(np.int64)
    off = np.zeros(count + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    steps = rng.standard_normal((int(off[-1]), 2), dtype=np.float32)
    steps[off[:-1]] = 0.0
    cs = np.cumsum(steps, axis=0, dtype=np.float64)
    del steps
    origin = rng.random((count, 2)) * 100.0
    cs -= np.repeat(cs[off[:-1]] - origin, lens, axis=0)
    host = cs.astype(np.float32)
    del cs
    pts = torch.from_numpy(host).to(device)
    out = (pts, torch.from_numpy(off).to(device), int(lens.max()))
    return out + ((host, off),) if keep_host else out


def make_requests(n: int, qlo: int, qhi: int, seed: int, measures=None):
    """n single-query requests: (measure, points, offsets)."""
    rng = np.random.default_rng(seed)
    names = list(measures or MEASURE_PARAMS)
    which = rng.integers(0, len(names), n)
    lens = rng.integers(qlo, qhi + 1, n)
    out = []
    for i in range(n):
        qp, qo = G.random_walks(1, [int(lens[i])], seed * 7919 + i)
        out.append((names[which[i]], qp, qo))
    return out


def _pct(a, q):
    return float(np.percentile(np.asarray(a), q)) if len(a) else None


def run_open_loop(server, requests, rate: float, k: int = 10, seed: int = 0, keep=(),
                  kept=None):
    """Submit ``requests`` at Poisson arrival times of ``rate`` per second and
    collect them.  Latency of a request = scheduled arrival -> results on the
    host (includes any lag of the submitting thread).  The results (ids,
    distances) of the requests whose indices are in ``keep`` are stored in
    the dict ``kept``."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(requests)))
    tickets = [None] * len(requests)
    submit_lag = np.zeros(len(requests))
    ready = threading.Semaphore(0)
    t0 = time.perf_counter() + 0.05

    def submitter():
        for i, (m, qp, qo) in enumerate(requests):
            target = t0 + arrivals[i]
            while True:
                now = time.perf_counter()
                if now >= target:
                    break
                if target - now > 1e-3:
                    time.sleep(min(target - now - 5e-4, 0.01))
            tickets[i] = server.submit(qp, qo, m, k, **MEASURE_PARAMS[m])
            submit_lag[i] = time.perf_counter() - target
            ready.release()

    th = threading.Thread(target=submitter)
    th.start()
    infos = []
    t_last = t0
    for i in range(len(requests)):
        ready.acquire()
        ids, dists, info = server.wait(tickets[i])
        if kept is not None and i in keep:
            kept[i] = (ids, dists)
        t_last = max(t_last, time.perf_counter())
        info["measure"] = requests[i][0]
        info["qlen"] = int(requests[i][2][-1])
        info["total_ms"] = info["latency_ms"] + submit_lag[i] * 1e3
        infos.append(info)
    th.join()
    span = t_last - t0
    return summarize(infos, span, offered=rate)


def run_closed_loop(server, requests, k: int = 10, flags: int = 0):
    """Submit everything at once (the queue keeps every slot busy): the
    server's capacity in requests/s.  ``flags``: TSIM_FLAG_* added to every
    request."""
    t0 = time.perf_counter()
    tickets = [server.submit(qp, qo, m, k, flags=flags, **MEASURE_PARAMS[m])
               for m, qp, qo in requests]
    infos = []
    for i, t in enumerate(tickets):
        _, _, info = server.wait(t)
        info["measure"] = requests[i][0]
        info["qlen"] = int(requests[i][2][-1])
        info["total_ms"] = info["latency_ms"]
        infos.append(info)
    return summarize(infos, time.perf_counter() - t0, offered=None)


def summarize(infos, span_s, offered):
    lat = [x["total_ms"] for x in infos]
    out = {
        "requests": len(infos),
        "offered_rps": offered,
        "achieved_rps": len(infos) / span_s if span_s > 0 else None,
        "p50_ms": _pct(lat, 50),
        "p99_ms": _pct(lat, 99),
        "mean_ms": float(np.mean(lat)) if lat else None,
        "queue_p50_ms": _pct([x["queue_ms"] for x in infos], 50),
        "queue_p99_ms": _pct([x["queue_ms"] for x in infos], 99),
        "device_ms_mean": float(np.mean([x["device_ms"] for x in infos])) if infos else None,
        "inflight_mean": float(np.mean([x["inflight_at_admit"] for x in infos])) if infos else None,
        "per_measure": {},
    }
    for m in MEASURE_PARAMS:
        sel = [x for x in infos if x["measure"] == m]
        if not sel:
            continue
        out["per_measure"][m] = {
            "requests": len(sel),
            "p50_ms": _pct([x["total_ms"] for x in sel], 50),
            "p99_ms": _pct([x["total_ms"] for x in sel], 99),
            "device_ms_p50": _pct([x["device_ms"] for x in sel], 50),
            "device_ms_p99": _pct([x["device_ms"] for x in sel], 99),
        }
    return out
