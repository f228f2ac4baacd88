"""Benchmark: exact batched DTW kNN on one GB300 (the batched uneven DTW workload).

Workload: 64 query trajectories x 16,384 candidate trajectories, 2-D float32
random walks (start uniform in [0,100)^2, N(0,1) steps), lengths uniform in
[64, 512]; DTW with squared-Euclidean cell cost, Sakoe-Chiba band of 10% of
the longer length, LB_Kim + LB_Keogh pruning, top-10 per query.  One step =
one exact kNN pass of all 64 queries over the device-resident database.

Reported: kNN queries/s of the batched form (device-resident inputs, CUDA
events), end-to-end queries/s through the host-pointer C-ABI entry point
(tsim_knn_host: H2D of the queries and D2H of ids/distances inside the timed
region), queries/s of the plain one-pair-per-launch form (same algorithm,
bounded sample), GCUPS, the roofline of the dominant kernel, measured error
against the FP64 CPU oracle, and the CPU baseline (oracle port, all cores and
one thread).

After the headline (N = 1 only), the line's ``workloads`` key carries the
other measured workloads, each with its own timed steps, clocks, roofline,
CPU baseline and parity against the FP64 oracle on a stated sample: the
small plain case of all five measures (8 x 1,024, L = 128, full DP; batched
vs plain one-pair-per-launch), LCSS + Frechet (256 x 65,536, lognormal
lengths), Hausdorff + Euclidean (1,024 x 262,144, Student-t steps) and the
serving loop (1M resident trajectories, Poisson arrivals at 2,000 req/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workloads all|none|name,...] [--workload NAME]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DTW kNN queries/s (batched, exact top-10, <=1e-5 rel err vs FP64)"
UNIT = "queries/s"
WORKLOAD = dict(workload="dtw_knn_batched_uneven", queries=64, candidates=16384, len_lo=64,
                len_hi=512, band_pct=10, cost="squared_euclidean", k=10, seed=2024)
DP_FLOPS_PER_CELL = 8  # 2 sub, mul, fma (2), 2 min, add
# dram__bytes_read.sum + dram__bytes_write.sum of the survivor-round DP launch
# of this workload (dp_wave_kernel, single stream), one ncu capture of
# `python -m cudaruntime1_gb300.profile_pass 1` on a GB300
SURVIVOR_DP_DRAM_BYTES = 11592448
L2_FLUSH_BYTES = 512 << 20


def make_data(w=WORKLOAD):
    from cudaruntime1_gb300 import datagen as G
    s = w["seed"]
    cl = G.uniform_lengths(w["candidates"], w["len_lo"], w["len_hi"], s)
    ql = G.uniform_lengths(w["queries"], w["len_lo"], w["len_hi"], s + 1)
    cp, co = G.random_walks(w["candidates"], cl, s + 2)
    qp, qo = G.random_walks(w["queries"], ql, s + 3)
    return qp, qo, cp, co


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def cpu_baseline(qp, qo, cp, co, w, min_seconds=10.0):
    """The oracle's exact pruned DTW kNN (the reference's CPU algorithm made
    exact and rectangular), all host threads, repeated to ~10 s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(ref=False)
    threads = O.num_threads()
    runs, t0 = 0, time.perf_counter()
    while True:
        ids, d, cells = O.dtw_knn_pruned(qp, qo, cp, co, w["k"], band_pct=w["band_pct"],
                                         cost=O.COST_SQEUCLID, nthreads=threads)
        runs += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or runs >= 50:
            break
    qps = runs * (len(qo) - 1) / el
    return {"value": qps, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{runs} full passes of {len(qo) - 1} queries x {len(co) - 1} candidates "
                      f"(oracle dtw_knn_pruned, FP64, OpenMP), {el:.1f} s"}, ids, d, cells


SAT_CANDIDATES = 2048  # every query against the first 2,048 candidates: 131,072 pairs


def dp_saturated(ctx, T, api, qpt, qot, maxq, cp, co, w, fp32_peak, stream, reps=5):
    """The FP32 DTW DP alone at saturation: every workload query against the
    first SAT_CANDIDATES candidates (the workload's shapes: lengths U[64,512],
    band 10 %, squared cost) through tsim_dp_pairs, with no threshold (no
    early abandon, no pruning).  Band cells (exact, tsim_band_cells) x 8
    flops over the CUDA-event time of the call on its stream."""
    import torch
    nq = len(qot) - 1
    nc = min(SAT_CANDIDATES, len(co) - 1)
    cpt = torch.from_numpy(cp[:co[nc]]).cuda()
    cot = torch.from_numpy(np.ascontiguousarray(co[:nc + 1])).cuda()
    qq, cc = np.meshgrid(np.arange(nq, dtype=np.int32), np.arange(nc, dtype=np.int32),
                         indexing="ij")
    pairs = torch.from_numpy(np.stack([qq.ravel(), cc.ravel()], 1).copy()).cuda()
    npairs = nq * nc
    out = torch.empty(npairs, dtype=torch.float32, device="cuda")
    maxc = int(np.max(np.diff(co[:nc + 1])))
    kw = dict(band_pct=w["band_pct"], cost=api.COST_SQEUCLID)
    db2 = T.Database(ctx, cp[:co[nc]], co[:nc + 1])
    cells = api.band_cells(ctx, db2, qpt.data_ptr(), qot.data_ptr(), nq, "dtw", **kw)
    db2.close()

    def timed(kernel):
        def call():
            api.dp_pairs(ctx, "dtw", 0, kernel, qpt.data_ptr(), qot.data_ptr(), maxq,
                         cpt.data_ptr(), cot.data_ptr(), maxc, pairs.data_ptr(), npairs,
                         out.data_ptr(), 0, **kw)

        call()
        torch.cuda.synchronize()
        ctx.counters(reset=True)
        ms = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            call()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        launches = ctx.counters(reset=True)["launches"] / reps
        return statistics.median(ms), ms, launches, out.cpu().numpy().copy()

    by_kernel, vals = {}, {}
    for name, kernel in (("warp_per_pair", 2), ("lane_per_pair", 5)):
        t, ms, launches, v = timed(kernel)
        vals[name] = v
        by_kernel[name] = {"ms": t, "ms_all": ms, "gcups": cells / (t * 1e6),
                           "launches_per_call": launches,
                           "frac": cells * DP_FLOPS_PER_CELL / (t * 1e-3) / 1e12 / fp32_peak
                           if fp32_peak else None}
    best = min(by_kernel, key=lambda k: by_kernel[k]["ms"])
    t = by_kernel[best]["ms"]
    tflops = cells * DP_FLOPS_PER_CELL / (t * 1e-3) / 1e12
    return {"pairs": npairs, "band_cells": int(cells), "kernel": best, "ms": t,
            "gcups": cells / (t * 1e6), "achieved": tflops, "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": tflops / fp32_peak if fp32_peak else None, "by_kernel": by_kernel,
            "values_bit_identical_across_kernels": bool(np.array_equal(
                vals["warp_per_pair"].view(np.uint32), vals["lane_per_pair"].view(np.uint32))),
            "what": f"{nq} queries x first {nc} candidates of the workload, FP32 DTW band "
                    f"{w['band_pct']}%, no threshold, tsim_dp_pairs per kernel, "
                    f"median of {reps} calls"}


def cpu_baseline_one_thread(qp, qo, cp, co, w, nsample=8):
    """The same CPU path on one thread, over the first ``nsample`` queries
    (the reference's original build ran its CPU code without OpenMP)."""
    import oracle as O
    qo_s = np.asarray(qo[:nsample + 1], np.int64)
    t0 = time.perf_counter()
    O.dtw_knn_pruned(qp[:qo_s[-1]], qo_s, cp, co, w["k"], band_pct=w["band_pct"],
                     cost=O.COST_SQEUCLID, nthreads=1)
    el = time.perf_counter() - t0
    return {"value": nsample / el, "unit": UNIT, "cores": 1,
            "sample": f"{nsample} queries x {len(co) - 1} candidates, {el:.2f} s"}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, local


def max_over_ranks(x: float) -> float:
    """The largest of the ranks' values (the replicas' timed regions): one
    all-reduce, on the device for NCCL, on the host for gloo."""
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


REF_BUDGET_S = 120.0  # wall time the reference arm's timed steps may take


def run_reference(args):
    """The CPU path (the oracle's exact pruned DTW kNN, all host threads):
    `warmup` untimed steps, then exactly `steps` timed ones.  A step is the
    workload's queries against the whole database, or, when `steps` full
    passes would exceed REF_BUDGET_S, a bounded sample of those queries
    (rotating through them), so the run stays within a few minutes."""
    rank, ws, _ = dist_init()
    if rank != 0:
        return
    qp, qo, cp, co = make_data()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(ref=False)
    threads = O.num_threads()
    nq, w = len(qo) - 1, WORKLOAD

    def step(q0, nb):
        sel = np.asarray(qo[q0:q0 + nb + 1]) - qo[q0]
        O.dtw_knn_pruned(qp[qo[q0]:qo[q0 + nb]], sel, cp, co, w["k"], band_pct=w["band_pct"],
                         cost=O.COST_SQEUCLID, nthreads=threads)

    t0 = time.perf_counter()
    step(0, nq)  # one full pass sizes the steps
    full_s = time.perf_counter() - t0
    nb = nq if args.steps * full_s <= REF_BUDGET_S else \
        max(1, min(nq, int(nq * REF_BUDGET_S / (args.steps * full_s))))
    for i in range(max(0, args.warmup - 1)):
        step((i * nb) % (nq - nb + 1), nb)
    done, t0 = 0, time.perf_counter()
    for i in range(args.steps):
        step((i * nb) % (nq - nb + 1), nb)
        done += nb
    el = time.perf_counter() - t0
    qps = done / el
    sample = (f"{args.steps} steps of {nb} of the {nq} queries x {len(co) - 1} candidates "
              f"(oracle dtw_knn_pruned, FP64, OpenMP), {el:.1f} s")
    base = {"value": qps, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
            **host_cpu()}
    line = {"impl": "reference", "metric": METRIC, "value": qps, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(WORKLOAD),
            "cpu_baseline": base,
            "e2e": {"value": qps, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# the other measured workloads: every measure, each over one device-resident
# database.  Each runs after the headline's timed region in the default bench
# run (the line's ``workloads`` key) and alone with ``--workload NAME``.  The
# CPU leg (the oracle's bound-pruned exact kNN, FP64, all host threads, on a
# stated sample of the queries) gives both the CPU baseline and the parity.
KNN_WORKLOADS = {
    "plain_small": dict(
        workload="plain_small_five_measures", queries=8, candidates=1024, len_lo=128, len_hi=128,
        lengths="fixed 128", step="normal", k=10, seed=11, cpu_queries=8, plain=True,
        runs=[("dtw", dict(band_pct=-1, cost=0), 0), ("lcss", dict(epsilon=0.5, delta=-1), 0),
              ("frechet", dict(), 0), ("hausdorff", dict(), 0), ("euclidean", dict(), 0)]),
    "lcss_frechet": dict(
        workload="lcss_frechet_256x65536", queries=256, candidates=65536,
        lengths="lognormal(ln 200, 0.6) clipped to [32, 1024]", step="normal", k=10, seed=23,
        cpu_queries=32, plain=False,
        runs=[("lcss", dict(epsilon=0.25, delta=20), 0), ("frechet", dict(), 8)]),
    "hausdorff_euclid": dict(
        workload="hausdorff_euclid_1024x262144", queries=1024, candidates=262144,
        lengths="Hausdorff: U[32, 256]; Euclidean: 256, 1% of candidates 2048, queries 2048",
        step="student_t(3)", k=10, seed=37, cpu_queries=32, plain=False,
        runs=[("hausdorff", dict(), 0), ("euclidean", dict(), 0)]),
}
# algorithmic flops (ops) per DP cell or point pair; compensation, masking
# and abandon checks are overhead, not counted
FLOPS_PER_UNIT = {"dtw": 8, "frechet": 7, "lcss": 6, "hausdorff": 6, "euclidean": 6}
REL_TOL = 1e-5


def host_cpu():
    """The host's CPU model, logical CPU count and architecture."""
    import platform
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            with open("/proc/cpuinfo") as f:
                for ln in f:
                    if ln.lower().startswith("model name"):
                        model = ln.split(":", 1)[1].strip()
                        break
        except OSError:
            pass
    return {"cpu_model": model or platform.processor() or "unknown", "nproc": os.cpu_count(),
            "arch": platform.machine()}


def step_stats(ms):
    """min / median / max of per-step times (ms)."""
    return {"min": float(min(ms)), "median": float(statistics.median(ms)), "max": float(max(ms))}


def knn_workload_data(name, w, measure):
    from cudaruntime1_gb300 import datagen as G
    s, nq, nc = w["seed"], w["queries"], w["candidates"]
    step = "student_t" if w["step"].startswith("student") else "normal"
    if name == "plain_small":
        ql, cl = np.full(nq, 128), np.full(nc, 128)
    elif name == "lcss_frechet":
        ql = G.lognormal_lengths(nq, np.log(200.0), 0.6, 32, 1024, s)
        cl = G.lognormal_lengths(nc, np.log(200.0), 0.6, 32, 1024, s + 1)
    elif measure == "hausdorff":
        ql, cl = G.uniform_lengths(nq, 32, 256, s), G.uniform_lengths(nc, 32, 256, s + 1)
    else:  # lock-step Euclidean: 256 points, 1% of the candidates 2048; queries 2048
        rng = np.random.default_rng(s + 2)
        cl = np.where(rng.random(nc) < 0.01, 2048, 256)
        ql = np.full(nq, 2048)
    cp, co = G.random_walks(nc, cl, s + 3, step=step)
    qp, qo = G.random_walks(nq, ql, s + 4, step=step)
    return qp, qo, cp, co


def profile_pass(ctx, step, flush, nsteps=3):
    """The request run on one stream with per-stage CUDA-event timers: stage
    times per step and the survivor round's refine (its launches' time and
    the cells / point pairs they computed).  In the timed region chunks of
    queries overlap on several streams, so no launch is separable there."""
    import tempfile
    tune_file = os.path.join(tempfile.mkdtemp(), "tuning.txt")
    ctx.save_tuning(tune_file)
    ctx.clear_tuning()
    ctx.set_concurrency(1)
    ctx.counters(reset=True)
    ctx.set_profiling(True)
    for _ in range(nsteps):
        flush.zero_()
        step()
    surv_cells = ctx.survivor_cells() / nsteps
    prof = ctx.counters(reset=True)
    ctx.set_profiling(False)
    ctx.set_concurrency(4)
    ctx.load_tuning(tune_file)
    stage_ms = {s: v / nsteps for s, v in prof["stage_ms"].items() if v > 0}
    calls = max(1.0, prof["stage_calls"]["dp_survivors"] / nsteps)
    return {"stage_ms": stage_ms,
            "dp_cells_per_step": prof["dp_cells"] / nsteps,
            "survivor_stage_calls": calls,
            "survivor_ms": stage_ms.get("dp_survivors", 0.0) / calls,
            "survivor_units": surv_cells / calls}


def refine_roofline(measure, prof, fp32_peak, hbm_peak):
    """Roofline of the survivor round's refine: algorithmic flops (and, for
    lock-step Euclidean, the candidate bytes it streams) per launch over its
    CUDA-event time.  The bound is the one the arithmetic intensity selects:
    DP cells and Hausdorff point pairs reuse each point across a row or a
    tile of points (FP32 issue), a lock-step Euclidean point pair reads one
    fresh 8-byte candidate point for its 6 flops (HBM)."""
    ms, units = prof["survivor_ms"], prof["survivor_units"]
    if not ms or not units:
        return None
    fl = FLOPS_PER_UNIT[measure]
    tflops = units * fl / (ms * 1e-3) / 1e12
    out = {"kernel": {"hausdorff": "hausdorff_refine_kernel", "euclidean": "euclid_refine_kernel"}
           .get(measure, f"dp_diag_kernel ({measure})") + ", survivor round",
           "unit_of_work": "point pair" if measure in ("hausdorff", "euclidean") else "DP cell",
           "units_per_launch": units, "launch_ms": ms, "flops_per_unit": fl,
           "fp32": {"achieved": tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                    "frac": tflops / fp32_peak if fp32_peak else None}}
    if measure == "euclidean":
        gbs = units * 8 / (ms * 1e-3) / 1e9
        out["hbm"] = {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s",
                      "frac": gbs / hbm_peak if hbm_peak else None,
                      "bytes_per_unit": 8}
        out["bound"] = "hbm"
    else:
        out["bound"] = "fp32"
    b = out[out["bound"]]
    out.update(achieved=b["achieved"], peak=b["peak"], unit=b["unit"], frac=b["frac"])
    return out


def knn_workload(args, name):
    """One of KNN_WORKLOADS on cuda:0: per measure, queries/s over exactly
    ``steps`` timed steps (device-resident inputs, L2 flushed before each),
    per-step spread, clocks, cell or point-pair rates, the survivor refine's
    roofline, the plain form where the workload asks for it, and the CPU leg
    (baseline and parity on a stated sample of the queries)."""
    import torch

    import cudaruntime1_gb300 as T
    from cudaruntime1_gb300 import api
    w = KNN_WORKLOADS[name]
    T.build()
    dev = 0
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    prev = torch.cuda.current_stream(dev)
    torch.cuda.set_stream(stream)
    ctx = T.Context(dev, stream.cuda_stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    fp32_peak = ctx.probe_fp32_tflops()
    hbm_peak = measured_peaks().get("hbm_gbs")
    k = w["k"]
    per = {}
    cache = {}
    total_launches = 0
    for measure, kw, flags in w["runs"]:
        key = measure if name == "hausdorff_euclid" else "all"  # one dataset per shape
        if key not in cache:
            cache = {key: knn_workload_data(name, w, measure)}
        qp, qo, cp, co = cache[key]
        nq = len(qo) - 1
        db = T.Database(ctx, cp, co)
        qpt = torch.from_numpy(qp).cuda()
        qot = torch.from_numpy(qo).cuda()
        ids = torch.empty(nq * k, dtype=torch.int32, device="cuda")
        dd = torch.empty(nq * k, dtype=torch.float32, device="cuda")
        d64 = torch.empty(nq * k, dtype=torch.float64, device="cuda")
        maxq = int(np.max(np.diff(qo)))
        tune = ctx.autotune(db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, measure, k, reps=3,
                            flags=flags, **kw)

        def step():
            api.knn_device(ctx, db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, ids.data_ptr(),
                           dd.data_ptr(), d64.data_ptr(), measure, k, flags=flags, **kw)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        ctx.counters(reset=True)
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        with ClockSampler(dev) as clk:
            for a, b in evs:
                flush.zero_()
                a.record(stream)
                step()
                b.record(stream)
            torch.cuda.synchronize()
        sms = [a.elapsed_time(b) for a, b in evs]
        ms = sum(sms)
        cnt = ctx.counters(reset=True)
        total_launches += cnt["launches"]
        r_ids = ids.cpu().numpy().reshape(nq, k)
        r_d = dd.cpu().numpy().reshape(nq, k).astype(np.float64)
        r_d64 = d64.cpu().numpy().reshape(nq, k)
        prof = profile_pass(ctx, step, flush)
        _, _, st = T.knn(ctx, db, qp, qo, measure, k, stats=True, flags=flags, **kw)
        pairwise = measure in ("hausdorff", "euclidean")
        units = cnt["dp_cells"] / args.steps
        res = {"queries_per_s": nq * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
               "step_ms": step_stats(sms), "gpu_launches_per_step": cnt["launches"] / args.steps,
               ("point_pairs_per_step" if pairwise else "dp_cells_per_step"): units,
               ("point_pairs_per_s" if pairwise else "gcups"):
                   (units / (ms / args.steps * 1e-3) if pairwise else
                    units / (ms / args.steps * 1e6)) if units else None,
               "funnel": {x: st[x] for x in ("pairs", "pairs_lb1", "pairs_lb2",
                                             "pairs_refined", "rescored", "rescored_fp64")},
               "stage_ms_single_stream": prof["stage_ms"],
               "roofline": refine_roofline(measure, prof, fp32_peak, hbm_peak),
               "autotune": tune, "params": dict(kw, flags=flags), "clocks": clk.summary()}
        if w["plain"]:
            T.knn(ctx, db, qp, qo, measure, k, flags=api.FLAG_PLAIN, **kw)
            t0 = time.perf_counter()
            p_ids, _, _ = T.knn(ctx, db, qp, qo, measure, k, flags=api.FLAG_PLAIN, **kw)
            res["plain_queries_per_s"] = nq / (time.perf_counter() - t0)
            res["batched_vs_plain"] = res["queries_per_s"] / res["plain_queries_per_s"]
            res["plain_ids_match"] = bool(np.array_equal(p_ids, r_ids))
        if not args.no_cpu:
            res["cpu_baseline"], res["parity"] = knn_cpu_leg(
                measure, kw, qp, qo, cp, co, k, w["cpu_queries"], r_ids, r_d, r_d64,
                brute=name == "plain_small")
        per[measure] = res
        db.close()
    ctx.close()
    torch.cuda.set_stream(prev)
    first = w["runs"][0][0]
    return {"metric": f"exact kNN queries/s per measure ({w['workload']})",
            "value": per[first]["queries_per_s"], "unit": "queries/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic",
            "config": {x: w[x] for x in w if x not in ("runs", "plain")},
            "value_measure": first, "per_measure": per, "gpu_launches": total_launches,
            "parity_ok": all(p.get("parity", {}).get("ok", True) for p in per.values()),
            "l2": "flushed before every timed step (512 MiB write)",
            "fp32_peak_tflops": fp32_peak}


def parity_of(measure, oids, od, r_ids, r_d, r_d64):
    """Ids bit-exact; LCSS counts exact; other distances within REL_TOL of
    the FP64 oracle (the FP32 outputs and the library's FP64-channel ones)."""
    n = len(oids)
    par = {"ids_bit_exact": bool(np.array_equal(oids, r_ids[:n]))}
    ok = par["ids_bit_exact"]
    if measure == "lcss":
        par["counts_exact"] = bool(np.array_equal(od, r_d[:n]))
        ok = ok and par["counts_exact"]
    else:
        fin = np.isfinite(od)
        same_inf = bool(np.array_equal(fin, np.isfinite(r_d[:n])))
        par["infinities_match"] = same_inf
        ok = ok and same_inf
        if fin.any():
            denom = np.maximum(od[fin], 1e-300)
            par["max_rel_err_f32"] = float(np.max(np.abs(r_d[:n][fin] - od[fin]) / denom))
            ok = ok and par["max_rel_err_f32"] <= REL_TOL
            if r_d64 is not None:
                par["max_rel_err_f64_output"] = float(np.max(np.abs(r_d64[:n][fin] - od[fin]) /
                                                             denom))
    par["rel_tol"] = REL_TOL
    par["ok"] = bool(ok)
    return par


def knn_cpu_leg(measure, kw, qp, qo, cp, co, k, nsample, r_ids, r_d, r_d64, brute=False):
    """The oracle's exact kNN (FP64, all host threads) on the first
    ``nsample`` queries: CPU queries/s and the parity of those queries.
    The bound-pruned search is the timed baseline; ``brute`` also times the
    brute force over every candidate (the plain method of the small
    workload) and checks against it."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build(ref=False)
    okw = dict(kw)
    if "epsilon" in okw:
        okw["eps"] = okw.pop("epsilon")
    nq = len(qo) - 1
    nsample = min(nsample, nq)
    qo_s = np.asarray(qo[:nsample + 1], np.int64)
    qp_s = qp[:qo_s[-1]]
    t0 = time.perf_counter()
    oids, od, ev = O.knn_pruned(measure, qp_s, qo_s, cp, co, k, evaluated=True, **okw)
    el = time.perf_counter() - t0
    cpu = host_cpu()
    base = {"value": nsample / el, "unit": "queries/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"{nsample} of {nq} queries x {len(co) - 1} candidates, oracle bound-pruned "
                      f"exact kNN (FP64, OpenMP, {O.num_threads()} threads), {el:.2f} s, "
                      f"{ev} exact evaluations", **cpu}
    if brute:
        t0 = time.perf_counter()
        bids, bd = O.knn(measure, qp_s, qo_s, cp, co, k, **okw)
        el = time.perf_counter() - t0
        base["brute_force"] = {"value": nsample / el, "unit": "queries/s",
                               "cores": O.num_threads(), "ids_equal_pruned": bool(
                                   np.array_equal(bids, oids))}
        oids, od = bids, bd
    par = parity_of(measure, oids, od, r_ids, r_d, r_d64)
    par.update(queries_checked=nsample, of_queries=nq,
               sample=f"queries 0..{nsample - 1} ({100.0 * nsample / nq:.1f}%)",
               oracle="brute force" if brute else "bound-pruned exact kNN (equals brute force)")
    return base, par


def run_knn_workload(args, name):
    print(json.dumps(knn_workload(args, name)))


SERVING = dict(workload="serving_mixed_measures", db_trajectories=1_000_000, db_len_lo=50,
               db_len_hi=500, query_len_lo=16, query_len_hi=2048, k=10, arrival="poisson",
               offered_rps=2000, measures="dtw,lcss,frechet,hausdorff,euclidean (uniform)",
               seed=77)


SHARED_REQUESTS = 300


def shared_thresholds_leg(T, S, ctx, db, reqs, w):
    """Repeated queries with and without TSIM_FLAG_SHARE_THRESHOLDS: each of
    ``reqs`` is served once (which fills the server's threshold cache when
    the flag is on), then the same requests again; the second pass's device
    time per request and capacity, with the flag against without, and
    whether the answers agree."""
    from cudaruntime1_gb300 import api
    out = {}
    answers = {}
    for name, flags in (("without", 0), ("with", api.FLAG_SHARE_THRESHOLDS)):
        with T.Server(ctx, db, slots=w["slots"], hbm_budget_bytes=w["hbm_budget_bytes"]) as srv:
            S.run_closed_loop(srv, reqs, w["k"], flags=flags)
            tickets = [srv.submit(qp, qo, m, w["k"], flags=flags, **S.MEASURE_PARAMS[m])
                       for m, qp, qo in reqs]
            t0 = time.perf_counter()
            res = [srv.wait(t) for t in tickets]
            span = time.perf_counter() - t0
            st = srv.stats()
        answers[name] = res
        dms = [info["device_ms"] for _, _, info in res]
        out[name] = {"device_ms_mean": float(np.mean(dms)), "device_ms_p50": float(np.median(dms)),
                     "capacity_rps": len(reqs) / span,
                     "shared_threshold_hits": st["shared_threshold_hits"]}
    out["device_ms_ratio"] = out["with"]["device_ms_mean"] / out["without"]["device_ms_mean"]
    out["answers_identical"] = all(
        np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        for a, b in zip(answers["without"], answers["with"]))
    out["what"] = (f"the first {len(reqs)} open-loop requests served twice on one server (closed "
                   "loop); figures are the second pass, whose queries all repeat")
    return out


def serving_workload(args):
    """Serving loop: a resident 1M-trajectory database, Poisson arrivals of
    single-query kNN requests of uniformly drawn measures and lengths,
    admitted by device-memory budget; p50/p99 latency and achieved rate,
    and the parity of the first request of each measure against the oracle
    on the same database."""
    import torch

    import cudaruntime1_gb300 as T
    from cudaruntime1_gb300 import serving as S
    T.build()
    w = dict(SERVING)
    w.update(slots=args.slots, hbm_budget_bytes=args.budget_gib << 30, seconds=args.serve_seconds)
    dev = 0
    torch.cuda.set_device(dev)
    ctx = T.Context(dev)
    t_gen = time.perf_counter()
    pts, off, max_len, (hpts, hoff) = S.device_random_walks(
        w["db_trajectories"], w["db_len_lo"], w["db_len_hi"], w["seed"], keep_host=True)
    torch.cuda.synchronize()
    db = T.Database(ctx, device_pts=pts.data_ptr(), device_off=off.data_ptr(),
                    count=w["db_trajectories"], max_len=max_len)
    gen_s = time.perf_counter() - t_gen
    n_open = int(w["offered_rps"] * w["seconds"])
    reqs = S.make_requests(n_open, w["query_len_lo"], w["query_len_hi"], w["seed"] + 1)
    warm = S.make_requests(max(3, args.warmup) * 5, w["query_len_lo"], w["query_len_hi"],
                           w["seed"] + 2)
    keep = {}
    for i, (m, _, _) in enumerate(reqs):  # the first request of each measure
        keep.setdefault(m, i)
    kept = {}
    with T.Server(ctx, db, slots=w["slots"], hbm_budget_bytes=w["hbm_budget_bytes"]) as srv:
        S.run_closed_loop(srv, warm, w["k"])
        closed = S.run_closed_loop(srv, reqs[: max(200, n_open // 4)], w["k"])
        with ClockSampler(dev) as clk:
            opened = S.run_open_loop(srv, reqs, w["offered_rps"], w["k"], seed=w["seed"] + 3,
                                     keep=set(keep.values()), kept=kept)
        st = srv.stats()
    shared = shared_thresholds_leg(T, S, ctx, db, reqs[:SHARED_REQUESTS], w)
    dev_bytes = db.device_bytes()
    db.close()
    ctx.close()
    del pts, off
    line = {"metric": "kNN requests/s served at 2,000 req/s offered (mixed measures, exact top-10)",
            "value": opened["achieved_rps"], "unit": "requests/s", "n_gpus": 1,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic", "config": w,
            "latency_ms": {"p50": opened["p50_ms"], "p99": opened["p99_ms"],
                           "mean": opened["mean_ms"]},
            "open_loop": opened, "closed_loop_capacity": closed, "server": st,
            "shared_thresholds": shared,
            "db_build_s": gen_s, "db_device_bytes": dev_bytes, "clocks": clk.summary()}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build(ref=False)
        par = {}
        for m, i in sorted(keep.items(), key=lambda x: x[1]):
            _, qp, qo = reqs[i]
            okw = dict(S.MEASURE_PARAMS[m])
            if "epsilon" in okw:
                okw["eps"] = okw.pop("epsilon")
            t0 = time.perf_counter()
            oids, od = O.knn_pruned(m, qp, qo, hpts, hoff, w["k"], **okw)
            el = time.perf_counter() - t0
            g_ids, g_d = kept[i]
            p = parity_of(m, oids, od, g_ids, g_d.astype(np.float64), None)
            p.update(request=i, query_len=int(qo[-1]), oracle_s=round(el, 2))
            par[m] = p
        line["parity"] = {"per_measure": par,
                          "sample": "the first request of each measure in the open loop, against "
                                    "the oracle's bound-pruned exact kNN over the same 1M "
                                    "trajectories (FP64)",
                          "ok": all(p["ok"] for p in par.values())}
    return line


def run_serving(args):
    print(json.dumps(serving_workload(args)))


REF_GPU = dict(workload="reference_semantics_1024", num_t=1024, n=128, m=128, seed=41,
               r=1000.0, noise=2.0, eps=0.5, top_k=10, euclid_k=50,
               data="the reference's generator shapes (CudaRuntime1/main.cu:12-64): uniform "
                    "[-1,1] steps clamped to [0,1000], candidates noisy resampled copies")


def ref_gpu_workload(args, reps=5):
    """The reference's own GPU kernels (compiled for sm_103a from its sources
    into oracle/_ref/*.cubin) beside this library's reference-semantics
    entry points, on the same inputs in the reference's semantics: num_t
    queries against num_t candidates, n = m = 128.  Kernel times only, CUDA
    events on one stream, median of ``reps``: for the reference its filter
    and refine kernels (its host top-10 and copies left out, which favours
    it), for this library the whole device call.  Outputs are compared."""
    import ctypes as C

    import torch

    import cudaruntime1_gb300 as T
    from cudaruntime1_gb300 import _lib, api
    from cudaruntime1_gb300 import datagen as G
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refgpu as RG
    w = dict(REF_GPU)
    why = RG.available()
    if why:
        return {"config": w, "unavailable": why}
    T.build()
    L = _lib.load()
    dev = 0
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    prev = torch.cuda.current_stream(dev)
    torch.cuda.set_stream(stream)
    ctx = T.Context(dev, stream.cuda_stream)
    num_t, n, m, K = w["num_t"], w["n"], w["m"], min(10, w["num_t"])
    t1 = G.ref_base_trajectories(num_t, n, w["seed"], r=w["r"])
    t2 = G.ref_similar_trajectories(t1, num_t, n, m, w["noise"], w["seed"] + 1, r=w["r"])
    d1 = torch.from_numpy(t1).cuda()
    d2 = torch.from_numpy(t2).cuda()
    D = RG.Driver()
    mods, fns = [], {}
    for meas in RG.KERNELS:
        mod, f = D.load(RG.cubin_path(meas))
        mods.append(mod)
        fns.update(f)
    st = stream.cuda_stream

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(statistics.median(ts))

    vp, ci, cf = C.c_void_p, C.c_int, C.c_float
    per = {}
    env = torch.from_numpy(RG.envelopes(t1, num_t, n)).cuda()
    mat = torch.empty(num_t * num_t, dtype=torch.float32, device="cuda")
    npairs = num_t * K
    res = torch.empty(npairs, dtype=torch.float32, device="cuda")
    ours = torch.empty(num_t, dtype=torch.float32, device="cuda")
    eps = w["eps"]
    grid_f = ((num_t + 15) // 16, (num_t + 15) // 16)
    refine_shape = {  # threads, shared bytes (dtw.cu:185-187, lcss.cu:205-206, frechet.cu:205-207)
        "dtw": ((min(n, m) // 32 + 1) * 32 if min(n, m) < 256 else 256, 3 * (n + 1) * 4),
        "lcss": (256, 3 * n * 4),
        "frechet": (min(min(n, m), 256), 3 * n * 4)}
    for meas in ("dtw", "lcss", "frechet"):
        filt, refine = (fns[x] for x in RG.KERNELS[meas])
        extra = [cf(eps)] if meas == "lcss" else []

        def run_filter():
            D.launch(filt, grid_f, (16, 16), 0, st, [vp(env.data_ptr()), vp(d2.data_ptr()),
                                                     vp(mat.data_ptr()), ci(num_t), ci(n),
                                                     ci(m)] + extra)
        ms_filter = timed(run_filter)
        pairs = torch.from_numpy(RG.top_pairs(mat.cpu().numpy(), num_t, K, meas == "lcss")).cuda()
        thr, smem = refine_shape[meas]

        def run_refine():
            D.launch(refine, (npairs,), (thr,), smem, st,
                     [vp(d1.data_ptr()), vp(d2.data_ptr()), vp(pairs.data_ptr()),
                      vp(res.data_ptr()), ci(npairs), ci(n), ci(m)] + extra)
        ms_refine = timed(run_refine)
        rv = res.cpu().numpy().reshape(num_t, K)
        ref_out = rv.max(1) if meas == "lcss" else rv.min(1)
        ms_ours = timed(lambda: api.ref_batch_device(ctx, meas, d1.data_ptr(), d2.data_ptr(),
                                                     num_t, n, m, ours.data_ptr(), eps))
        ov = ours.cpu().numpy()
        per[meas] = {"ref_gpu_filter_ms": ms_filter, "ref_gpu_refine_ms": ms_refine,
                     "ref_gpu_kernels_ms": ms_filter + ms_refine, "ours_ms": ms_ours,
                     "speedup_vs_ref_gpu_kernels": (ms_filter + ms_refine) / ms_ours,
                     "ref_gpu_refine_pairs": npairs,
                     "outputs_bit_equal": int(np.sum(ov.view(np.uint32) == ref_out.view(np.uint32))),
                     "outputs_of": num_t,
                     "max_abs_diff": float(np.max(np.abs(ov.astype(np.float64) - ref_out)))}
    # Hausdorff and Euclidean from given candidates (the bounding-box nearest
    # neighbours that stand in for the reference's R-tree query)
    for meas, kk in (("hausdorff", w["top_k"]), ("euclidean", w["euclid_k"])):
        cand = torch.empty(num_t * kk, dtype=torch.int32, device="cuda")
        _lib.check(L.tsim_mbr_knn(ctx.h, vp(d1.data_ptr()), num_t, n, vp(d2.data_ptr()), num_t,
                                  m, kk, vp(cand.data_ptr())))
        outr = torch.empty(num_t, dtype=torch.float32, device="cuda")
        if meas == "hausdorff":
            f = fns["hausdorff_tiled_rtree_kernel"]
            ms_ref = timed(lambda: D.launch(
                f, (num_t,), (256,), 0, st,
                [vp(d1.data_ptr()), ci(num_t), ci(n), vp(d2.data_ptr()), ci(num_t), ci(m),
                 vp(cand.data_ptr()), ci(kk), vp(outr.data_ptr())]))
            ms_ours = timed(lambda: _lib.check(L.tsim_hausdorff_cands(
                ctx.h, vp(d1.data_ptr()), num_t, n, vp(d2.data_ptr()), num_t, m,
                vp(cand.data_ptr()), kk, vp(ours.data_ptr()))))
        else:
            off = torch.arange(0, num_t * kk + 1, kk, dtype=torch.int32, device="cuda")
            f = fns["euclidean_rtree_csr_kernel_global"]
            ms_ref = timed(lambda: D.launch(
                f, (num_t,), (256,), 0, st,
                [vp(d1.data_ptr()), vp(d2.data_ptr()), vp(cand.data_ptr()), vp(off.data_ptr()),
                 vp(outr.data_ptr()), ci(num_t), ci(n)]))
            ms_ours = timed(lambda: _lib.check(L.tsim_euclid_cands(
                ctx.h, vp(d1.data_ptr()), vp(d2.data_ptr()), vp(cand.data_ptr()),
                vp(off.data_ptr()), num_t, n, num_t * kk, vp(ours.data_ptr()))))
        rv, ov = outr.cpu().numpy(), ours.cpu().numpy()
        per[meas] = {"ref_gpu_kernel_ms": ms_ref, "ours_ms": ms_ours,
                     "speedup_vs_ref_gpu_kernel": ms_ref / ms_ours, "candidates_per_query": kk,
                     "outputs_bit_equal": int(np.sum(ov.view(np.uint32) == rv.view(np.uint32))),
                     "outputs_of": num_t,
                     "max_rel_diff": float(np.max(np.abs(ov.astype(np.float64) - rv) /
                                                  np.maximum(np.abs(rv), 1e-30)))}
    for mod in mods:
        D.L.cuModuleUnload(mod)
    ctx.close()
    torch.cuda.set_stream(prev)
    return {"metric": "kernel ms, reference's own GPU kernels vs this library, reference "
                      "semantics", "config": w, "per_measure": per,
            "timing": f"CUDA events on one stream, median of {reps}; reference: its kernels only "
                      "(host envelopes, top-10 and copies excluded); ours: the whole device call"}


DEFAULT_WORKLOADS = ("plain_small", "lcss_frechet", "hausdorff_euclid", "serving", "ref_gpu")


def extra_workloads(args):
    """The workloads other than the headline, after its timed region: each
    its own measurement (errors recorded, not raised, so the headline line
    is always printed)."""
    import traceback
    names = DEFAULT_WORKLOADS if args.workloads == "all" else \
        tuple(x for x in args.workloads.split(",") if x and x != "none")
    out = {}
    for nm in names:
        t0 = time.perf_counter()
        try:
            if nm == "serving":
                out[nm] = serving_workload(args)
            elif nm == "ref_gpu":
                out[nm] = ref_gpu_workload(args)
            else:
                out[nm] = knn_workload(args, nm)
        except Exception as e:  # recorded in the line; the traceback goes to stderr
            traceback.print_exc()
            out[nm] = {"error": f"{type(e).__name__}: {e}"}
        out[nm]["wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--kernels-only", action="store_true",
                    help="only the warm-up and timed steps (for profiler launch lists)")
    ap.add_argument("--save-tuning", default=None,
                    help="write the autotuner's choices to this file")
    ap.add_argument("--load-tuning", default=None,
                    help="take the launch choices from this file instead of autotuning "
                         "(profiled runs: the autotuner would time the profiler's serialised launches)")
    ap.add_argument("--workload", default="dtw_knn_batched_uneven",
                    choices=["dtw_knn_batched_uneven", "serving", "ref_gpu"] + list(KNN_WORKLOADS))
    ap.add_argument("--serve-seconds", type=float, default=5.0)
    ap.add_argument("--slots", type=int, default=32)
    ap.add_argument("--budget-gib", type=int, default=8)
    ap.add_argument("--workloads", default="all",
                    help="after the headline: 'all' (" + ",".join(DEFAULT_WORKLOADS) + "), "
                         "'none', or a comma list; measured on one GPU, reported under the "
                         "line's 'workloads' key")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "ref_gpu":
        return print(json.dumps(ref_gpu_workload(args)))
    if args.workload in KNN_WORKLOADS:
        return run_knn_workload(args, args.workload)

    import torch
    import torch.distributed as dist

    import cudaruntime1_gb300 as T
    from cudaruntime1_gb300 import api

    rank, ws, local = dist_init()
    dev = local
    torch.cuda.set_device(dev)
    T.build()
    # an explicit stream: the library, torch's events and the L2 flush all use it
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    w = WORKLOAD
    qp, qo, cp, co = make_data()
    nq, k = len(qo) - 1, w["k"]
    ctx = T.Context(dev, stream.cuda_stream)
    db = T.Database(ctx, cp, co)
    qpt = torch.from_numpy(qp).to(f"cuda:{dev}")
    qot = torch.from_numpy(qo).to(f"cuda:{dev}")
    ids = torch.empty(nq * k, dtype=torch.int32, device=f"cuda:{dev}")
    dd = torch.empty(nq * k, dtype=torch.float32, device=f"cuda:{dev}")
    d64 = torch.empty(nq * k, dtype=torch.float64, device=f"cuda:{dev}")
    maxq = int(np.max(np.diff(qo)))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")
    kw = dict(band_pct=w["band_pct"], cost=api.COST_SQEUCLID)

    def step():
        api.knn_device(ctx, db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, ids.data_ptr(),
                       dd.data_ptr(), d64.data_ptr(), "dtw", k, **kw)

    # launch choices (rows per lane-group, concurrent query chunks) picked by
    # the autotuner on this request before anything is timed
    if args.load_tuning:
        ctx.load_tuning(args.load_tuning)
        tune = {"loaded": args.load_tuning}
    else:
        tune = ctx.autotune(db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, "dtw", k, reps=5, **kw)
    if args.save_tuning:
        ctx.save_tuning(args.save_tuning)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ctx.counters(reset=True)

    # ---- timed region: device-resident inputs, L2 flushed before every step
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        torch.cuda.nvtx.range_push("timed_steps")  # profilers capture this range alone
        for s, e in evs:
            flush.zero_()
            s.record(stream)
            step()
            e.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
    step_ms = [s.elapsed_time(e) for s, e in evs]
    total_ms = sum(step_ms)
    cnt = ctx.counters(reset=True)
    launches = cnt["launches"]
    # clock evidence over a longer stretch of the same steps (the timed
    # region lasts only a few tens of ms: a few nvidia-smi samples)
    soak_n = max(50, int(round(1000.0 / max(total_ms / args.steps, 1e-3))))
    with ClockSampler(dev) as soak_clk:
        s0 = torch.cuda.Event(enable_timing=True)
        s1 = torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        for _ in range(soak_n):
            step()
        s1.record(stream)
        torch.cuda.synchronize()
    soak = {"steps": soak_n, "ms_per_step": s0.elapsed_time(s1) / soak_n,
            "l2": "not flushed between steps", "clocks": soak_clk.summary()}
    ctx.counters(reset=True)
    if ws > 1:
        total_ms = max_over_ranks(total_ms)
    value = ws * nq * args.steps / (total_ms / 1e3)
    res_ids = ids.cpu().numpy().reshape(nq, k)
    res_d64 = d64.cpu().numpy().reshape(nq, k)
    if args.kernels_only:
        print(json.dumps({"kernels_only": True, "ms_per_step": total_ms / args.steps,
                          "launches": launches}))
        return

    # ---- per-stage device times (CUDA events on the launching stream); the
    # chunks of a request overlap on child streams in the timed region, so
    # per-kernel durations are taken with one stream
    import tempfile
    tune_file = os.path.join(tempfile.mkdtemp(), "tuning.txt")
    ctx.save_tuning(tune_file)
    ctx.clear_tuning()
    ctx.set_concurrency(1)
    ctx.set_profiling(True)
    prof_steps = 5
    for _ in range(prof_steps):
        flush.zero_()
        step()
    surv_cells = ctx.survivor_cells() / prof_steps
    prof = ctx.counters(reset=True)
    ctx.set_profiling(False)
    ctx.set_concurrency(4)
    ctx.load_tuning(tune_file)
    stage_ms = {s: v / prof_steps for s, v in prof["stage_ms"].items() if v > 0}
    dp_cells = prof["dp_cells"] / prof_steps
    # the dominant kernel: the survivor round's DP launch (one per step here)
    surv_calls = max(1.0, prof["stage_calls"]["dp_survivors"] / prof_steps)
    surv_ms = stage_ms.get("dp_survivors", 0.0) / surv_calls
    surv_cells_launch = surv_cells / surv_calls
    _, _, funnel = T.knn(ctx, db, qp, qo, "dtw", k, stats=True, **kw)
    band_cells = api.band_cells(ctx, db, qpt.data_ptr(), qot.data_ptr(), nq, "dtw",
                                band_pct=w["band_pct"])
    fp32_peak = ctx.probe_fp32_tflops()
    sat = dp_saturated(ctx, T, api, qpt, qot, maxq, cp, co, w, fp32_peak, stream)

    # ---- plain form: one DP pair per kernel launch, bounded sample of queries
    nplain = 4
    qo_p = qo[:nplain + 1]
    qp_p = qp[:qo_p[-1]]
    ids_p, _, _ = T.knn(ctx, db, qp_p, qo_p, "dtw", k, flags=api.FLAG_PLAIN, **kw)  # warm
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ids_p, _, st_p = T.knn(ctx, db, qp_p, qo_p, "dtw", k, flags=api.FLAG_PLAIN, **kw)
    plain_s = time.perf_counter() - t0
    plain_qps = nplain / plain_s
    plain_ok = bool(np.array_equal(ids_p, res_ids[:nplain]))
    ctx.counters(reset=True)

    # ---- end to end: host arrays through the C-ABI host entry point
    h2d = qp.nbytes + qo.nbytes
    d2h = nq * k * (4 + 4)
    for _ in range(3):
        T.knn(ctx, db, qp, qo, "dtw", k, stats=False, **kw)
    e2e_ms = 0.0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e_ids, _, _ = T.knn(ctx, db, qp, qo, "dtw", k, stats=False, **kw)
        e2e_ms += (time.perf_counter() - t0) * 1e3
    e2e_ok = bool(np.array_equal(e_ids, res_ids))
    e2e_qps = ws * nq * args.steps / (e2e_ms / 1e3)

    line = None
    if rank == 0:
        # ---- CPU baseline and parity against the FP64 oracle on this workload
        base = None
        ids_match = None
        max_rel = None
        if not args.no_cpu:
            base, oids, od, ocells = cpu_baseline(qp, qo, cp, co, w)
            base.update(host_cpu())
            base["one_thread"] = cpu_baseline_one_thread(qp, qo, cp, co, w)
            ids_match = bool(np.array_equal(oids, res_ids))
            fin = np.isfinite(od)
            max_rel = float(np.max(np.abs(res_d64[fin] - od[fin]) / np.maximum(od[fin], 1e-300)))
            dd_f = dd.cpu().numpy().reshape(nq, k).astype(np.float64)
            max_rel = max(max_rel, float(np.max(np.abs(dd_f[fin] - od[fin]) / od[fin])))
        peaks = measured_peaks()
        step_s = total_ms / args.steps / 1e3
        dominant = max(stage_ms, key=stage_ms.get) if stage_ms else "dp"
        achieved = (surv_cells_launch * DP_FLOPS_PER_CELL / (surv_ms * 1e-3) / 1e12
                    if surv_ms else 0.0)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(w, l2="flushed before every timed step (512 MiB write)",
                           inputs_bytes=int(cp.nbytes + co.nbytes + qp.nbytes)),
            "gcups": dp_cells / (step_s * 1e9),
            "gcups_effective": band_cells / (step_s * 1e9),
            "dp_cells_per_step": dp_cells, "band_cells_per_step": band_cells,
            "survivor_cell_frac": dp_cells / band_cells if band_cells else None,
            "stage_ms": stage_ms, "dominant_stage": dominant,
            "funnel": {x: funnel[x] for x in ("pairs", "pairs_lb1", "pairs_lb2", "pairs_refined",
                                              "rescored", "rescored_fp64")},
            "autotune": tune,
            "plain": {"value": plain_qps, "unit": UNIT, "sample_queries": nplain,
                      "ids_match_batched": plain_ok},
            "batched_vs_plain": value / plain_qps if plain_qps else None,
            "parity": {"ids_bit_exact_vs_fp64_oracle": ids_match, "max_rel_err": max_rel},
            "dp_saturated": sat,
            "roofline": {
                "kernel": "dp_wave_kernel<PolDtwSq,R>, survivor round (FP32 band-relative "
                          "anti-diagonal DTW, a warp per pair)",
                "bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak if fp32_peak else None,
                "traffic": SURVIVOR_DP_DRAM_BYTES, "traffic_unit": "bytes per launch (ncu)",
                "peak_source": "measured FP32 FMA probe kernel on this GPU (tsim_probe_fp32_tflops)",
                "flops_per_cell": DP_FLOPS_PER_CELL, "cells_per_launch": surv_cells_launch,
                "launch_ms": surv_ms,
                "timing": "CUDA events around the launch on its stream, single-stream "
                          "profiling pass of the same workload after the timed region"},
            "cpu_baseline": base,
            "e2e": {"value": e2e_qps, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ids_match_device_path": e2e_ok},
            "gpu_launches": int(launches),
            "gpu_launches_per_step": launches / args.steps,
            "step_ms": step_stats(step_ms),
            "clocks": clk.summary(),
            "clock_soak": soak,
            "hbm_peak_gbs": peaks.get("hbm_gbs"),
        }
    db.close()
    ctx.close()
    if line is not None:
        if ws == 1 and args.workloads != "none":
            line["workloads"] = extra_workloads(args)
        print(json.dumps(line))
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
