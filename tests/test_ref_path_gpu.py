"""GPU parity of the reference-named entry points against the reference's
own CPU results (golden fixtures) and the oracle's restatement: bit-exact."""
import os

import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_batch.npz")

FN = {
    "dtw": lambda T, t1, t2, n, m, num_t, eps: T.launch_dtw_batch_gpu_knn(t1, t2, num_t, n, m),
    "lcss": lambda T, t1, t2, n, m, num_t, eps: T.launch_lcss_batch_gpu_wavefront_knn(
        t1, t2, num_t, n, m, eps),
    "frechet": lambda T, t1, t2, n, m, num_t, eps: T.launch_frechet_batch_gpu_wavefront(
        t1, t2, num_t, n, m),
}


def _bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("measure", ["dtw", "lcss", "frechet"])
def test_golden_fixtures_bit_exact(tsim, cuda_ctx, measure):
    z = np.load(GOLD)
    for ci in range(int(z["ncases"][0])):
        num_t, n, m = (int(v) for v in z[f"c{ci}_meta"])
        eps = float(z[f"c{ci}_eps"][0])
        got, ms = FN[measure](tsim, z[f"c{ci}_t1"], z[f"c{ci}_t2"], n, m, num_t, eps)
        assert ms > 0.0
        want = z[f"c{ci}_{measure}"]
        assert np.array_equal(_bits(got), _bits(want)), (measure, ci, got, want)


@pytest.mark.parametrize("measure", ["dtw", "lcss", "frechet"])
@pytest.mark.parametrize("shape", [(64, 128, 128), (40, 100, 120), (33, 250, 200), (1, 7, 9),
                                   (20, 520, 480)])
def test_random_shapes_bit_exact(tsim, cuda_ctx, oracle, measure, shape):
    num_t, n, m = shape
    t1 = G.ref_base_trajectories(num_t, n, 7 + n, r=300.0)
    t2 = G.ref_similar_trajectories(t1, num_t, n, m, 2.0, 9 + m, r=300.0)
    got, _ = FN[measure](tsim, t1, t2, n, m, num_t, 0.5)
    want = oracle.ref_batch(measure, t1, t2, n, m, eps=0.5)
    assert np.array_equal(_bits(got), _bits(want))


def test_random_walks_square_1024(tsim, cuda_ctx, oracle):
    """The parity case of the small plain workload, square as the reference
    API requires: 1,024 x 1,024 trajectories of length 128."""
    pts, _ = G.random_walks(1024, 128, 21)
    pts2, _ = G.random_walks(1024, 128, 22)
    for meas in ("dtw", "lcss", "frechet"):
        got, _ = FN[meas](tsim, pts, pts2, 128, 128, 1024, 0.5)
        want = oracle.ref_batch(meas, pts, pts2, 128, 128, eps=0.5)
        assert np.array_equal(_bits(got), _bits(want)), meas


def test_hausdorff_given_candidates(tsim, cuda_ctx, oracle):
    num_t1, num_t2, n, m = 30, 45, 70, 90
    t1 = G.ref_base_trajectories(num_t1, n, 31, r=200.0)
    t2 = G.ref_base_trajectories(num_t2, m, 32, r=200.0)
    cand = oracle.mbr_knn(t1, n, t2, m, 10)
    got, ms = tsim.launch_hausdorff_rtree_gpu(t1, num_t1, n, t2, num_t2, m, cand, 10)
    want = oracle.ref_hausdorff_cands(t1, n, t2, m, cand)
    assert np.array_equal(_bits(got), _bits(want))
    # against the FP64 definition
    for i in range(0, num_t1, 7):
        best = min(oracle.pair("hausdorff", t1[i * n:(i + 1) * n], t2[c * m:(c + 1) * m])
                   for c in cand[i * 10:(i + 1) * 10])
        assert abs(got[i] - best) <= 1e-6 * max(1.0, best)


def test_hausdorff_pipeline(tsim, cuda_ctx, oracle):
    num_t, n, m = 60, 100, 120
    t1 = G.ref_base_trajectories(num_t, n, 41, r=1000.0)
    t2 = G.ref_similar_trajectories(t1, num_t, n, m, 2.0, 42, r=1000.0)
    got, ms = tsim.run_hausdorff_rtree_gpu_pipeline(t1, num_t, n, t2, num_t, m, 10)
    cand = oracle.mbr_knn(t1, n, t2, m, 10)
    want = oracle.ref_hausdorff_cands(t1, n, t2, m, cand)
    assert np.array_equal(_bits(got), _bits(want))
    # fewer candidates than top_k: padded like the reference (hausdorff_rtree.cpp:66-68)
    got3, _ = tsim.run_hausdorff_rtree_gpu_pipeline(t1[:3 * n], 3, n, t2[:2 * m], 2, m, 10)
    want3 = oracle.ref_hausdorff_cands(t1[:3 * n], n, t2[:2 * m], m, oracle.mbr_knn(t1[:3 * n], n, t2[:2 * m], m, 10))
    assert np.array_equal(_bits(got3), _bits(want3))


def test_euclidean_csr_and_pipeline(tsim, cuda_ctx, oracle):
    num_t, n = 200, 96
    t1 = G.ref_base_trajectories(num_t, n, 51, r=100.0)
    t2 = G.ref_similar_trajectories(t1, num_t, n, n, 2.0, 52, r=100.0)
    rng = np.random.default_rng(3)
    counts = rng.integers(0, 30, num_t)
    off = np.zeros(num_t + 1, np.int32)
    off[1:] = np.cumsum(counts)
    cand = rng.integers(0, num_t, off[-1]).astype(np.int32)
    got, _ = tsim.execute_rtree_csr_kernel_on_gpu(t1, t2, cand, off, num_t, n, int(off[-1]))
    want = oracle.ref_euclid_cands(t1, t2, n, cand, off)
    assert np.array_equal(_bits(got), _bits(want))
    got2, _ = tsim.launch_euclidean_batch_gpu_rtree_exact(t1, t2, num_t, n)
    k = min(50, num_t)
    c2 = oracle.mbr_knn(t1, n, t2, n, k)
    want2 = oracle.ref_euclid_cands(t1, t2, n, c2, np.arange(0, num_t * k + 1, k, dtype=np.int32))
    assert np.array_equal(_bits(got2), _bits(want2))
