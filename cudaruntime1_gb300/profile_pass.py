"""Fixed launch sequences for profiler captures: no autotuning, no timing, no
graph replay, one chunk on a single stream.

    python -m cudaruntime1_gb300.profile_pass [passes]
        exact-kNN passes of the batched DTW workload (per pass: the seed
        round, round 1, the survivor round and the re-score, each an R-chain
        of anti-diagonal passes, then the selections)
    python -m cudaruntime1_gb300.profile_pass --serving
        one 16-query DTW request against the serving workload's resident
        1,000,000-trajectory database (lengths U[50, 500], about 2.4 GB on
        the device), where the filter kernels' reads exceed L2
    python -m cudaruntime1_gb300.profile_pass --dp-one KERNEL
        three tsim_dp_pairs calls on one 512 x 486 DTW pair (band 10 %)
        with the given kernel (2: warp per pair, 4: two warps, 5: a lane per
        pair, 6: band-relative): one pair's latency
    python -m cudaruntime1_gb300.profile_pass --dp-saturated KERNEL
        one tsim_dp_pairs call on every batched-workload query against its
        first 2,048 candidates (131,072 FP32 DTW pairs, no threshold)
    python -m cudaruntime1_gb300.profile_pass --lcss-frechet
        one LCSS and one Frechet exact-kNN request of the 256 x 65,536
        workload (lognormal lengths) on one stream
    python -m cudaruntime1_gb300.profile_pass --hausdorff-euclid MEASURE [NQ]
        one exact-kNN request (MEASURE hausdorff or euclidean) of the
        1,024 x 262,144 workload on one stream, or of its first NQ queries
"""
from __future__ import annotations

import os
import sys

import numpy as np


def dp_pairs_case(kernel, saturated):
    import torch

    import cudaruntime1_gb300 as T
    from bench import make_data
    from cudaruntime1_gb300 import api
    from cudaruntime1_gb300 import datagen as G
    T.build()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = T.Context(0, stream.cuda_stream)
    if saturated:
        qp, qo, cp, co = make_data()
        nq, nc = len(qo) - 1, 2048
        co = np.ascontiguousarray(co[:nc + 1])
        cp = cp[:co[-1]]
        qq, cc = np.meshgrid(np.arange(nq, dtype=np.int32), np.arange(nc, dtype=np.int32),
                             indexing="ij")
        pairs = np.stack([qq.ravel(), cc.ravel()], 1).astype(np.int32)
        calls = 1
    else:
        qp, qo = G.random_walks(1, np.array([512]), 1)
        cp, co = G.random_walks(1, np.array([486]), 2)
        pairs = np.zeros((1, 2), np.int32)
        calls = 3
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda()
         for k, v in dict(qp=qp, qo=qo, cp=cp, co=co, pr=pairs).items()}
    out = torch.empty(len(pairs), dtype=torch.float32, device="cuda")
    for _ in range(calls):
        api.dp_pairs(ctx, "dtw", 0, kernel, d["qp"].data_ptr(), d["qo"].data_ptr(),
                     int(np.max(np.diff(qo))), d["cp"].data_ptr(), d["co"].data_ptr(),
                     int(np.max(np.diff(co))), d["pr"].data_ptr(), len(pairs), out.data_ptr(), 0,
                     band_pct=10, cost=api.COST_SQEUCLID)
    torch.cuda.synchronize()
    print("ok", float(out[:8].sum()))
    ctx.close()


def lcss_frechet_case():
    import torch

    import cudaruntime1_gb300 as T
    from bench import KNN_WORKLOADS, knn_workload_data
    from cudaruntime1_gb300 import api
    T.build()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = T.Context(0, stream.cuda_stream)
    ctx.set_concurrency(1)
    w = KNN_WORKLOADS["lcss_frechet"]
    qp, qo, cp, co = knn_workload_data("lcss_frechet", w, "lcss")
    db = T.Database(ctx, cp, co)
    qpt, qot = torch.from_numpy(qp).cuda(), torch.from_numpy(qo).cuda()
    nq, maxq, k = len(qo) - 1, int(np.max(np.diff(qo))), w["k"]
    ids = torch.empty(nq * k, dtype=torch.int32, device="cuda")
    dd = torch.empty(nq * k, dtype=torch.float32, device="cuda")
    d64 = torch.empty(nq * k, dtype=torch.float64, device="cuda")
    for measure, kw, flags in w["runs"]:
        api.knn_device(ctx, db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, ids.data_ptr(),
                       dd.data_ptr(), d64.data_ptr(), measure, k, flags=flags | api.FLAG_NO_GRAPH,
                       **kw)
    torch.cuda.synchronize()
    print("ok", ids[:k].tolist())
    db.close()
    ctx.close()


def hausdorff_euclid_case(measure, nq_use):
    import torch

    import cudaruntime1_gb300 as T
    from bench import KNN_WORKLOADS, knn_workload_data
    from cudaruntime1_gb300 import api
    T.build()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = T.Context(0, stream.cuda_stream)
    ctx.set_concurrency(1)
    w = KNN_WORKLOADS["hausdorff_euclid"]
    qp, qo, cp, co = knn_workload_data("hausdorff_euclid", w, measure)
    db = T.Database(ctx, cp, co)
    qpt, qot = torch.from_numpy(qp).cuda(), torch.from_numpy(qo).cuda()
    nq = nq_use if nq_use > 0 else len(qo) - 1
    maxq, k = int(np.max(np.diff(qo))), w["k"]
    ids = torch.empty(nq * k, dtype=torch.int32, device="cuda")
    dd = torch.empty(nq * k, dtype=torch.float32, device="cuda")
    api.knn_device(ctx, db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, ids.data_ptr(),
                   dd.data_ptr(), 0, measure, k, flags=api.FLAG_NO_GRAPH)
    torch.cuda.synchronize()
    print("ok", ids[:k].tolist())
    db.close()
    ctx.close()


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    for flag in ("--dp-one", "--dp-saturated"):
        if flag in argv:
            return dp_pairs_case(int(argv[argv.index(flag) + 1]), flag == "--dp-saturated")
    if "--lcss-frechet" in argv:
        return lcss_frechet_case()
    if "--hausdorff-euclid" in argv:
        i = argv.index("--hausdorff-euclid")
        rest = argv[i + 1:]
        return hausdorff_euclid_case(rest[0], int(rest[1]) if len(rest) > 1 else 0)
    serving = "--serving" in argv
    argv = [x for x in argv if x != "--serving"]
    passes = int(argv[0]) if argv else 1
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch

    import cudaruntime1_gb300 as T
    from bench import SERVING, WORKLOAD, make_data  # the workloads bench.py measures
    from cudaruntime1_gb300 import api
    from cudaruntime1_gb300 import datagen as G

    T.build()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = T.Context(0, stream.cuda_stream)
    ctx.set_concurrency(1)
    k = WORKLOAD["k"]
    if serving:
        from cudaruntime1_gb300 import serving as S
        w = SERVING
        pts, off, max_len = S.device_random_walks(w["db_trajectories"], w["db_len_lo"],
                                                  w["db_len_hi"], w["seed"])
        torch.cuda.synchronize()
        db = T.Database(ctx, device_pts=pts.data_ptr(), device_off=off.data_ptr(),
                        count=w["db_trajectories"], max_len=max_len)
        nq = 16
        qp, qo = G.random_walks(nq, G.uniform_lengths(nq, w["query_len_lo"], w["query_len_hi"],
                                                      w["seed"] + 5), w["seed"] + 6)
    else:
        qp, qo, cp, co = make_data()
        db = T.Database(ctx, cp, co)
        nq = len(qo) - 1
    qpt = torch.from_numpy(qp).cuda()
    qot = torch.from_numpy(qo).cuda()
    ids = torch.empty(nq * k, dtype=torch.int32, device="cuda")
    dd = torch.empty(nq * k, dtype=torch.float32, device="cuda")
    maxq = int(np.max(np.diff(qo)))
    for _ in range(passes):
        api.knn_device(ctx, db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, ids.data_ptr(),
                       dd.data_ptr(), 0, "dtw", k, band_pct=WORKLOAD["band_pct"],
                       cost=api.COST_SQEUCLID, flags=api.FLAG_NO_GRAPH)
    torch.cuda.synchronize()
    print("ok", ids[:k].tolist())
    db.close()
    ctx.close()


if __name__ == "__main__":
    main()
