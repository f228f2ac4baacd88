"""The CPU oracle, pinned before anything is checked against it.

* its reference-semantics restatement equals the reference's own CPU code
  (tests/golden fixtures made from CudaRuntime1/dtw.cpp, lcss.cpp,
  frechet.cpp, and the compiled reference itself when present);
* its FP64 measures satisfy known answers derived from the definitions;
* its pruned DTW kNN equals its brute-force kNN.
"""
import os

import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_batch.npz")


def _cases():
    z = np.load(GOLD)
    for ci in range(int(z["ncases"][0])):
        num_t, n, m = (int(v) for v in z[f"c{ci}_meta"])
        yield ci, z, num_t, n, m, float(z[f"c{ci}_eps"][0])


@pytest.mark.parametrize("measure", ["dtw", "lcss", "frechet"])
def test_restatement_matches_golden(oracle, measure):
    for ci, z, num_t, n, m, eps in _cases():
        got = oracle.ref_batch(measure, z[f"c{ci}_t1"], z[f"c{ci}_t2"], n, m, eps=eps)
        want = z[f"c{ci}_{measure}"]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (ci, got, want)


@pytest.mark.parametrize("measure", ["dtw", "lcss", "frechet"])
def test_restatement_matches_compiled_reference(oracle, measure):
    if oracle.ref_lib() is None:
        pytest.skip("reference checkout not present: pinned by the golden fixtures instead")
    rng = np.random.default_rng(5)
    for trial in range(4):
        num_t, n, m = int(rng.integers(1, 40)), int(rng.integers(1, 60)), int(rng.integers(1, 60))
        t1 = G.ref_base_trajectories(num_t, n, 200 + trial, r=100.0)
        t2 = G.ref_similar_trajectories(t1, num_t, n, m, 2.0, 300 + trial, r=100.0)
        a = oracle.ref_batch(measure, t1, t2, n, m, eps=0.5)
        b = oracle.ref_batch(measure, t1, t2, n, m, eps=0.5, use_ref=True)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_known_answers(oracle):
    pts, off = G.random_walks(3, [20, 20, 1], 9)
    a = pts[off[0]:off[1]]
    single = pts[off[2]:off[3]]
    for meas in ("dtw", "frechet", "hausdorff", "euclidean"):
        assert oracle.pair(meas, a, a) == 0.0
    # single points: every measure is the point distance
    p, q = single, single + np.float32([3.0, 4.0])
    assert oracle.pair("dtw", p, q, cost=oracle.COST_EUCLID) == 5.0
    assert oracle.pair("dtw", p, q, cost=oracle.COST_SQEUCLID) == 25.0
    assert oracle.pair("frechet", p, q) == 5.0
    assert oracle.pair("hausdorff", p, q) == 5.0
    assert oracle.pair("euclidean", p, q) == 5.0
    # LCSS of a trajectory with itself is its length; shifted beyond eps is 0
    assert oracle.pair("lcss", a, a, eps=0.5) == len(a)
    assert oracle.pair("lcss", a, a + np.float32(1.0), eps=0.5) == 0
    # a translated copy: Frechet and Euclidean are the shift length (up to the
    # float32 rounding of the shifted coordinates, ~1e-5 at magnitude 100)
    sh = np.float32([0.6, 0.8])
    assert abs(oracle.pair("frechet", a, a + sh) - 1.0) < 1e-4
    assert oracle.pair("hausdorff", a, a + sh) <= 1.0 + 1e-4
    assert abs(oracle.pair("euclidean", a, a + sh) - np.sqrt(len(a))) < 1e-3
    # symmetry
    b = pts[off[1]:off[2]]
    for meas in ("dtw", "frechet", "hausdorff"):
        assert oracle.pair(meas, a, b) == oracle.pair(meas, b, a)
    assert oracle.pair("lcss", a, b, eps=2.0, delta=3) == oracle.pair("lcss", b, a, eps=2.0, delta=3)
    # a band only removes paths
    assert oracle.pair("dtw", a, b, band_pct=10) >= oracle.pair("dtw", a, b)


def test_band_geometry(oracle):
    for n, m in [(64, 512), (512, 64), (300, 300), (2, 1000), (1, 5), (5, 1), (100, 101)]:
        w = oracle.band_w(n, m, 10)
        assert w == -(-10 * max(n, m) // 100)
        prev = (-1, -1)
        for i in range(n):
            lo, hi = oracle.band_row(i, n, m, w)
            if lo <= hi:
                assert lo >= prev[0] and hi >= prev[1]
                prev = (lo, hi)
        assert oracle.band_row(0, n, m, w)[0] == 0
        assert oracle.band_row(n - 1, n, m, w)[1] == m - 1


def test_pruned_dtw_knn_equals_brute_force(oracle):
    ql = G.uniform_lengths(6, 20, 60, 1)
    cl = G.uniform_lengths(300, 20, 60, 2)
    qp, qo = G.random_walks(6, ql, 3)
    cp, co = G.random_walks(300, cl, 4)
    for band, cost in [(10, 0), (-1, 0), (25, 1)]:
        ids_b, d_b = oracle.knn("dtw", qp, qo, cp, co, 7, band_pct=band, cost=cost)
        ids_p, d_p, cells = oracle.dtw_knn_pruned(qp, qo, cp, co, 7, band_pct=band, cost=cost)
        assert np.array_equal(ids_b, ids_p)
        assert np.array_equal(d_b, d_p)
        assert cells > 0


def test_grid_hausdorff_matches_brute_force(oracle):
    pts, off = G.random_walks(12, [40, 55, 30, 70, 12, 80, 44, 9, 60, 33, 25, 50], 8)
    for i in range(0, 12, 2):
        a, b = pts[off[i]:off[i + 1]], pts[off[i + 1]:off[i + 2]]
        d1 = oracle.directed_hausdorff_grid(a, b, 0.0)
        d2 = oracle.directed_hausdorff_grid(b, a, d1)
        want = oracle.pair("hausdorff", a, b)
        assert abs(np.sqrt(np.float64(d2)) - want) <= 1e-6 * max(1.0, want)


def test_knn_ties_break_by_index(oracle):
    pts, off = G.random_walks(1, 30, 11)
    q = pts.copy()
    db = np.concatenate([q + 5.0, q, q, q + 5.0])
    doff = np.arange(0, 5 * 30, 30, dtype=np.int64)
    ids, d = oracle.knn("dtw", q, np.array([0, 30]), db, doff, 4)
    assert list(ids[0]) == [1, 2, 0, 3]
    assert d[0][0] == d[0][1] == 0.0 and d[0][2] == d[0][3]


@pytest.mark.parametrize("measure,kw", [
    ("dtw", dict(band_pct=10)), ("dtw", dict(band_pct=-1, cost=1)),
    ("lcss", dict(eps=0.5, delta=5)), ("lcss", dict(eps=1.0)),
    ("frechet", {}), ("hausdorff", {}), ("euclidean", {})])
def test_pruned_knn_equals_brute_force(oracle, measure, kw):
    """The pruned exact kNN that checks parity against large databases gives
    the brute force's ids and values, ties and infinite values included."""
    ql = G.uniform_lengths(7, 10, 70, 21)
    cl = G.uniform_lengths(400, 10, 70, 22)
    qp, qo = G.random_walks(7, ql, 23, start_range=30.0)
    cp, co = G.random_walks(400, cl, 24, start_range=30.0)
    # duplicates of the first candidates (index ties) and a copy of query 0
    # (distance 0 / a full LCSS count)
    dup = cp[co[0]:co[3]]
    q0 = qp[qo[0]:qo[1]]
    cp = np.concatenate([cp, dup, dup, q0])
    co = np.concatenate([co, co[-1] + np.cumsum(np.diff(co[:4])),
                         co[-1] + co[3] + np.cumsum(np.diff(co[:4])),
                         [co[-1] + 2 * co[3] + len(q0)]]).astype(np.int64)
    for k in (1, 8):
        ids_b, d_b = oracle.knn(measure, qp, qo, cp, co, k, **kw)
        ids_p, d_p, ev = oracle.knn_pruned(measure, qp, qo, cp, co, k, evaluated=True, **kw)
        assert np.array_equal(ids_b, ids_p), (measure, k)
        assert np.array_equal(d_b, d_p), (measure, k)
        assert ev <= len(qo[:-1]) * (len(co) - 1)
    if measure == "euclidean":  # many candidates longer than the queries: +inf
        assert np.isinf(oracle.knn(measure, qp, qo, cp, co, 300)[1]).any()
        ids_b, d_b = oracle.knn(measure, qp, qo, cp, co, 300)
        ids_p, d_p = oracle.knn_pruned(measure, qp, qo, cp, co, 300)
        assert np.array_equal(ids_b, ids_p) and np.array_equal(d_b, d_p)
