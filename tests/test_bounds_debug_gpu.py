"""The bounds-checked build (libtsim_debug.so, TSIM_DEBUG_BOUNDS): every
shared-memory index of the DP kernels (row-group, band-relative, lane per
pair, striped) and the pairwise kernels is checked against its array, and
an index outside is counted instead of used.  The kernels run over every
DP kernel choice, every measure, pruned and brute-force kNN and the
given-candidate Hausdorff / Euclidean calls; not one index may fall
outside.  This stands in for a memory checker, which cannot run on this
GPU pool.  The run goes in a child process with TSIM_LIB pointing at the
debug library."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes as C, json, sys
import numpy as np, torch
sys.path.insert(0, ROOT)
import cudaruntime1_gb300 as T
from cudaruntime1_gb300 import _lib, api, datagen as G
L = _lib.load()
ctx = T.Context(0)
rng = np.random.default_rng(5)
# tsim_dp_pairs: every kernel, measure and precision
ql = G.uniform_lengths(10, 2, 400, 1); cl = G.uniform_lengths(60, 2, 400, 2)
qp, qo = G.random_walks(10, ql, 3); cp, co = G.random_walks(60, cl, 4)
pairs = np.stack([rng.integers(0, 10, 500), rng.integers(0, 60, 500)], 1).astype(np.int32)
d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
     dict(qp=qp, qo=qo, cp=cp, co=co, pr=pairs).items()}
o32 = torch.empty(500, device="cuda"); o64 = torch.empty(500, dtype=torch.float64, device="cuda")
for measure, kw in (("dtw", dict(band_pct=10, cost=0)), ("dtw", dict(band_pct=-1, cost=1)),
                    ("lcss", dict(epsilon=0.5, delta=7)), ("frechet", {})):
    for kernel in range(7):
        for prec in ((0,) if measure == "lcss" else (0, 1, 2)):
            api.dp_pairs(ctx, measure, prec, kernel, d["qp"].data_ptr(), d["qo"].data_ptr(),
                         int(ql.max()), d["cp"].data_ptr(), d["co"].data_ptr(), int(cl.max()),
                         d["pr"].data_ptr(), 500, o32.data_ptr(), o64.data_ptr(), **kw)
torch.cuda.synchronize()
# exact kNN, every measure, pruned and brute force
cp, co = G.random_walks(2500, G.uniform_lengths(2500, 16, 300, 7), 8)
qp, qo = G.random_walks(8, G.uniform_lengths(8, 16, 300, 9), 10)
db = T.Database(ctx, cp, co)
for measure, kw in (("dtw", dict(band_pct=10)), ("lcss", dict(epsilon=0.5, delta=9)),
                    ("frechet", {}), ("hausdorff", {}), ("euclidean", {})):
    for flags in (api.FLAG_ALWAYS_PRUNE, api.FLAG_NO_PRUNE, 0):
        T.knn(ctx, db, qp, qo, measure, 10, stats=False, flags=flags, **kw)
db.close()
# given-candidate Hausdorff and Euclidean (reference semantics)
t1 = G.ref_base_trajectories(64, 96, 11, r=500.0)
t2 = G.ref_similar_trajectories(t1, 64, 96, 96, 2.0, 12, r=500.0)
T.run_hausdorff_rtree_gpu_pipeline(t1, 64, 96, t2, 64, 96, 10)
T.launch_euclidean_batch_gpu_rtree_exact(t1, t2, 64, 96)
torch.cuda.synchronize()
n, f = C.c_int64(), C.c_int64()
assert L.tsim_debug_bounds_violations(C.byref(n), C.byref(f)) == 0
print(json.dumps({"violations": n.value, "first": f.value}))
"""


def test_no_shared_memory_index_out_of_bounds(tsim):
    from cudaruntime1_gb300 import buildlib as B
    lib = B.build(debug_bounds=True)
    env = dict(os.environ, TSIM_LIB=lib)
    r = subprocess.run([sys.executable, "-c", "ROOT = %r\n" % ROOT + CHILD], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["violations"] == 0, out
