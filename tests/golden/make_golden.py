"""Generate tests/golden/ref_batch.npz: inputs and outputs of the reference's
own CPU functions (CudaRuntime1/dtw.cpp launch_dtw_batch_cpu, lcss.cpp
launch_lcss_batch_cpu, frechet.cpp launch_frechet_batch_cpu), compiled from
the reference sources by oracle/Makefile (`make -C oracle ref`).

Run from the repository root:  python tests/golden/make_golden.py
The reference checkout is needed only here; the fixture travels without it.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from cudaruntime1_gb300 import datagen as G  # noqa: E402

CASES = [  # (num_t, n, m, seed, r, eps) -- reference-style clamped walks
    (24, 40, 50, 101, 100.0, 0.5),
    (17, 33, 21, 102, 100.0, 0.5),
    (12, 64, 64, 103, 1000.0, 0.5),
    (10, 9, 13, 104, 50.0, 1.0),
    (3, 1, 5, 105, 100.0, 0.5),
    (11, 25, 1, 106, 100.0, 0.5),
]


def main():
    O.build(ref=True)
    if O.ref_lib() is None:
        raise SystemExit("reference CPU library not built (needs the reference checkout)")
    out = {}
    for ci, (num_t, n, m, seed, r, eps) in enumerate(CASES):
        t1 = G.ref_base_trajectories(num_t, n, seed, r=r)
        t2 = G.ref_similar_trajectories(t1, num_t, n, m, 2.0, seed + 1000, r=r)
        out[f"c{ci}_t1"] = t1
        out[f"c{ci}_t2"] = t2
        out[f"c{ci}_meta"] = np.array([num_t, n, m], np.int64)
        out[f"c{ci}_eps"] = np.array([eps], np.float32)
        for meas in ("dtw", "lcss", "frechet"):
            out[f"c{ci}_{meas}"] = O.ref_batch(meas, t1, t2, n, m, eps=eps, use_ref=True)
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_batch.npz"),
                        ncases=np.array([len(CASES)]), **out)
    print("wrote ref_batch.npz with", len(CASES), "cases")


if __name__ == "__main__":
    main()
