"""Error paths, exercised without faulting the GPU.

tsim_debug_fail_allocations makes the library's next device or pinned-host
allocations fail on the host, as if the GPU were out of memory: the call that
meets one must return TSIM_ERR_OUT_OF_MEMORY and leave its context, its
database and the reference-named entry points usable -- the next call, with
the injection disarmed, returns the same answer as a context that never saw
a failure.  (The reference's host code exits on the first CUDA error,
CudaRuntime1/common.cuh's CHECK; the reference-named entry points keep that
unless TSIM_COMPAT_NO_EXIT is set.)

tsim_debug_set_canary fills every scratch reservation with 0xff bytes (NaN
floats, -1 integers) before a call's kernels run: no result may change, so
no kernel reads scratch before writing it.

tsim_debug_set_wait_limit(0) makes every bounded device-side wait on a bulk
copy run out at once (nothing is faulted or hung: the copies complete, the
kernel just stops waiting for them, reads global memory instead and waits
for them before it exits).  The synchronising call reports TSIM_ERR_TIMEOUT;
its context stays usable.
"""
import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu
OOM = 3
TIMEOUT = 4


def _data(seed, nc=800, nq=3, lo=20, hi=120):
    cp, co = G.random_walks(nc, G.uniform_lengths(nc, lo, hi, seed), seed + 1)
    qp, qo = G.random_walks(nq, G.uniform_lengths(nq, lo, hi, seed + 2), seed + 3)
    return cp, co, qp, qo


@pytest.fixture
def lib(tsim):
    L = tsim._lib.load()
    yield L
    L.tsim_debug_fail_allocations(0, 0)
    L.tsim_debug_set_canary(0)
    L.tsim_debug_set_wait_limit(-1)


def test_arena_allocation_failure_leaves_context_usable(tsim, lib):
    cp, co, qp, qo = _data(11)
    _, _, qp2, qo2 = _data(17, nq=40)
    with tsim.Context(0) as ref:
        dref = tsim.Database(ref, cp, co)
        want_small = tsim.knn(ref, dref, qp, qo, "dtw", 10, stats=False, band_pct=10)[:2]
        want_big = tsim.knn(ref, dref, qp2, qo2, "dtw", 10, stats=False, band_pct=10)[:2]
        dref.close()
    # a fresh context's first request allocates its pinned and device staging
    # and its scratch (and its chunks' child contexts): the first, second or
    # third of those allocations fails
    for skip in (0, 1, 2):
        with tsim.Context(0) as ctx:
            db = tsim.Database(ctx, cp, co)
            assert lib.tsim_debug_fail_allocations(skip, 1) == 0
            with pytest.raises(tsim._lib.TsimError) as err:
                tsim.knn(ctx, db, qp2, qo2, "dtw", 10, stats=False, band_pct=10)
            assert err.value.status == OOM, str(err.value)
            lib.tsim_debug_fail_allocations(0, 0)
            for qq, oo, want in ((qp2, qo2, want_big), (qp, qo, want_small)):
                got = tsim.knn(ctx, db, qq, oo, "dtw", 10, stats=False, band_pct=10)[:2]
                assert np.array_equal(got[0], want[0]), skip
                assert np.array_equal(got[1].view(np.uint32), want[1].view(np.uint32)), skip
            db.close()


def test_database_allocation_failure(tsim, lib):
    cp, co, qp, qo = _data(23)
    with tsim.Context(0) as ctx:
        for skip in range(4):  # points, offsets, then the summaries
            lib.tsim_debug_fail_allocations(skip, 1)
            with pytest.raises(tsim._lib.TsimError) as err:
                tsim.Database(ctx, cp, co)
            assert err.value.status == OOM
        lib.tsim_debug_fail_allocations(0, 0)
        db = tsim.Database(ctx, cp, co)
        ids, d, _ = tsim.knn(ctx, db, qp, qo, "frechet", 10, stats=False)
        db.close()
    with tsim.Context(0) as ref:
        dref = tsim.Database(ref, cp, co)
        ids2, d2, _ = tsim.knn(ref, dref, qp, qo, "frechet", 10, stats=False)
        dref.close()
    assert np.array_equal(ids, ids2) and np.array_equal(d.view(np.uint32), d2.view(np.uint32))


def test_reference_entry_point_buffer_failure(tsim, lib, monkeypatch):
    """The reference-named launch function with a failing buffer allocation:
    with TSIM_COMPAT_NO_EXIT it reports the error and returns NaN instead of
    exiting; the next call (injection off) returns the right values."""
    monkeypatch.setenv("TSIM_COMPAT_NO_EXIT", "1")
    t1 = G.ref_base_trajectories(64, 40, 5, r=200.0)
    t2 = G.ref_similar_trajectories(t1, 64, 40, 48, 2.0, 6, r=200.0)
    want, _ = tsim.launch_dtw_batch_gpu_knn(t1, t2, 64, 40, 48)
    big1 = G.ref_base_trajectories(512, 64, 7, r=200.0)
    big2 = G.ref_similar_trajectories(big1, 512, 64, 72, 2.0, 8, r=200.0)
    want_big, _ = tsim.launch_dtw_batch_gpu_knn(big1, big2, 512, 64, 72)
    # a still larger call must grow the cached buffers: make that fail
    huge1 = G.ref_base_trajectories(2048, 64, 9, r=200.0)
    huge2 = G.ref_similar_trajectories(huge1, 2048, 64, 72, 2.0, 10, r=200.0)
    lib.tsim_debug_fail_allocations(0, 1)
    got, _ = tsim.launch_dtw_batch_gpu_knn(huge1, huge2, 2048, 64, 72)
    assert np.isnan(got).all()
    lib.tsim_debug_fail_allocations(0, 0)
    got, _ = tsim.launch_dtw_batch_gpu_knn(big1, big2, 512, 64, 72)
    assert np.array_equal(got.view(np.uint32), want_big.view(np.uint32))
    got, _ = tsim.launch_dtw_batch_gpu_knn(t1, t2, 64, 40, 48)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("measure,kw", [("dtw", dict(band_pct=10)), ("lcss", dict(epsilon=0.5, delta=8)),
                                        ("frechet", {}), ("hausdorff", {}), ("euclidean", {})])
def test_scratch_canary_changes_nothing(tsim, lib, measure, kw):
    cp, co, qp, qo = _data(31, nc=2500, nq=6, lo=16, hi=200)
    with tsim.Context(0) as ctx:
        db = tsim.Database(ctx, cp, co)
        runs = {}
        for canary in (0, 1):
            lib.tsim_debug_set_canary(canary)
            for flags in (0, tsim.api.FLAG_ALWAYS_PRUNE, tsim.api.FLAG_NO_PRUNE):
                # no graph replay: every call reserves (and fills) its scratch
                ids, d, _ = tsim.knn(ctx, db, qp, qo, measure, 10, stats=False,
                                     flags=flags | tsim.api.FLAG_NO_GRAPH, **kw)
                runs[(canary, flags)] = (ids, d)
        lib.tsim_debug_set_canary(0)
        for flags in (0, tsim.api.FLAG_ALWAYS_PRUNE, tsim.api.FLAG_NO_PRUNE):
            a, b = runs[(0, flags)], runs[(1, flags)]
            assert np.array_equal(a[0], b[0]), (measure, flags)
            assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32)), (measure, flags)
        db.close()


def test_bounded_wait_timeout_is_reported(tsim, lib):
    """The DTW O(length) stage waits (boundedly) for its bulk copies of
    candidate points -- made for a database larger than L2, here 50,000
    trajectories of 240-300 points (108 MB).  With the limit at 0 every wait
    runs out: the call returns TSIM_ERR_TIMEOUT, and the next one (limit
    restored) returns the same answer as before."""
    cp, co, qp, qo = _data(41, nc=50000, nq=6, lo=240, hi=300)
    assert cp.nbytes > 100 * (1 << 20)
    fl = tsim.api.FLAG_ALWAYS_PRUNE | tsim.api.FLAG_NO_GRAPH
    with tsim.Context(0) as ctx:
        db = tsim.Database(ctx, cp, co)
        want = tsim.knn(ctx, db, qp, qo, "dtw", 10, stats=True, band_pct=10, flags=fl)
        assert want[2]["pairs_lb2"] > 0  # the stage ran
        assert lib.tsim_debug_set_wait_limit(0) == 0
        with pytest.raises(tsim._lib.TsimError) as err:
            tsim.knn(ctx, db, qp, qo, "dtw", 10, stats=True, band_pct=10, flags=fl)
        assert err.value.status == TIMEOUT, str(err.value)
        lib.tsim_debug_set_wait_limit(-1)
        got = tsim.knn(ctx, db, qp, qo, "dtw", 10, stats=True, band_pct=10, flags=fl)
        assert np.array_equal(got[0], want[0])
        assert np.array_equal(got[1].view(np.uint32), want[1].view(np.uint32))
        db.close()
