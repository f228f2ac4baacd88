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
"""
from __future__ import annotations

import os
import sys

import numpy as np


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
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
