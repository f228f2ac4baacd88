"""One exact-kNN pass of the batched DTW workload on a single stream, for
profiler captures: no autotuning, no timing, no graph replay, so the launch
sequence is fixed (per pass: the seed round, round 1, the survivor round and
the re-score, each an R-chain of anti-diagonal passes, then the selections).

    python -m cudaruntime1_gb300.profile_pass [passes]
"""
from __future__ import annotations

import os
import sys

import numpy as np


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    passes = int(argv[0]) if argv else 1
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch

    import cudaruntime1_gb300 as T
    from bench import WORKLOAD, make_data  # the workload bench.py measures
    from cudaruntime1_gb300 import api

    T.build()
    qp, qo, cp, co = make_data()
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = T.Context(0, stream.cuda_stream)
    ctx.set_concurrency(1)
    db = T.Database(ctx, cp, co)
    nq, k = len(qo) - 1, WORKLOAD["k"]
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
