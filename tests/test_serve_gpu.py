"""Serving loop (tsim_server_*): requests of mixed measures and lengths,
admitted by device-memory budget and run concurrently on stream slots, give
the same results as the same requests run alone, and the FP64 oracle's ids."""
import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu

PARAMS = {
    "dtw": dict(band_pct=10, cost=0),
    "lcss": dict(epsilon=0.25, delta=20),
    "frechet": dict(),
    "hausdorff": dict(),
    "euclidean": dict(),
}


def _requests(n, seed, lo=16, hi=300):
    rng = np.random.default_rng(seed)
    names = list(PARAMS)
    out = []
    for i in range(n):
        nq = int(rng.integers(1, 4))
        lens = rng.integers(lo, hi + 1, nq)
        qp, qo = G.random_walks(nq, lens, seed * 1000 + i)
        out.append((names[i % len(names)], qp, qo))
    return out


@pytest.fixture(scope="module")
def served_db(tsim, cuda_ctx):
    cp, co = G.random_walks(3000, G.uniform_lengths(3000, 20, 200, 41), 42)
    db = tsim.Database(cuda_ctx, cp, co)
    yield cp, co, db
    db.close()


def test_mixed_requests_match_alone(tsim, cuda_ctx, oracle, served_db):
    cp, co, db = served_db
    reqs = _requests(30, 5)
    k = 10
    alone = [tsim.knn(cuda_ctx, db, qp, qo, m, k, stats=False, **PARAMS[m]) for m, qp, qo in reqs]
    with tsim.Server(cuda_ctx, db, slots=8, hbm_budget_bytes=512 << 20) as srv:
        tickets = [srv.submit(qp, qo, m, k, **PARAMS[m]) for m, qp, qo in reqs]
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["peak_in_flight"] >= 2, st  # requests really overlapped
    for (m, qp, qo), (ia, da, _), (ig, dg, info) in zip(reqs, alone, got):
        assert info["status"] == 0
        assert np.array_equal(ia, ig), m
        assert np.array_equal(da, dg), m  # bit-identical alone and in the mix
    # and the ids are the exact kNN ids (a sample of each measure)
    seen = set()
    for (m, qp, qo), (ig, dg, _) in zip(reqs, got):
        if m in seen:
            continue
        seen.add(m)
        kw = dict(PARAMS[m])
        if "epsilon" in kw:
            kw["eps"] = kw.pop("epsilon")
        want_ids, _ = oracle.knn(m, qp, qo, cp, co, k, **kw)
        assert np.array_equal(ig, want_ids), m


def test_budget_limits_requests_in_flight(tsim, cuda_ctx, served_db):
    cp, co, db = served_db
    reqs = []  # equal shapes, so that the pool holds about two at a time
    for i, m in enumerate(list(PARAMS) * 2):
        qp, qo = G.random_walks(2, np.full(2, 200), 900 + i)
        reqs.append((m, qp, qo))
    k = 10
    need = max(tsim.knn_scratch_bytes(db, m, len(qo) - 1, int(np.max(np.diff(qo))), k,
                                      **PARAMS[m]) for m, qp, qo in reqs)
    budget = int(2.5 * (need + (64 << 10)))  # room for about two requests
    alone = [tsim.knn(cuda_ctx, db, qp, qo, m, k, stats=False, **PARAMS[m]) for m, qp, qo in reqs]
    with tsim.Server(cuda_ctx, db, slots=8, hbm_budget_bytes=budget) as srv:
        tickets = [srv.submit(qp, qo, m, k, **PARAMS[m]) for m, qp, qo in reqs]
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs)
    assert st["peak_scratch_bytes"] <= st["budget_bytes"]
    # the pool held a few requests at a time, never all of them (a batch of
    # requests needs a little less scratch than the requests apart)
    assert 1 <= st["peak_in_flight"] <= 3 < len(reqs), st
    for (ia, da, _), (ig, dg, _) in zip(alone, got):
        assert np.array_equal(ia, ig) and np.array_equal(da, dg)


def test_oversize_request_rejected_and_server_survives(tsim, cuda_ctx, served_db):
    cp, co, db = served_db
    qp, qo = G.random_walks(64, np.full(64, 100), 3)
    with tsim.Server(cuda_ctx, db, slots=2, hbm_budget_bytes=1 << 20) as srv:
        with pytest.raises(tsim.api._lib.TsimError) as e:
            srv.submit(qp, qo, "dtw", 10, **PARAMS["dtw"])
        assert e.value.status == tsim.api._lib.TSIM_ERR_BUDGET
        assert srv.stats()["rejected"] == 1
    # a small request still runs on a server whose pool fits it
    qp1, qo1 = G.random_walks(1, [50], 4)
    with tsim.Server(cuda_ctx, db, slots=2, hbm_budget_bytes=64 << 20) as srv:
        ids, d, info = srv.wait(srv.submit(qp1, qo1, "frechet", 5))
        assert info["status"] == 0 and ids.shape == (1, 5)


def test_wait_timeout_and_destroy_with_pending(tsim, cuda_ctx, served_db):
    cp, co, db = served_db
    reqs = _requests(30, 11, 1000, 2000)
    srv = tsim.Server(cuda_ctx, db, slots=1, hbm_budget_bytes=256 << 20)
    tickets = [srv.submit(qp, qo, m, 10, **PARAMS[m]) for m, qp, qo in reqs]
    r = srv.wait(tickets[-1], timeout_ms=0)  # queued behind 29 others
    assert r is None
    first = srv.wait(tickets[0])
    assert first[2]["status"] == 0
    srv.close()  # finishes the request in flight, fails the queued ones


def test_shared_thresholds_same_answers(tsim, cuda_ctx, oracle, served_db):
    """TSIM_FLAG_SHARE_THRESHOLDS: the server keeps each completed query's
    final pruning threshold and starts a later identical query (same
    parameters and points) from it.  Repeated requests then report shared
    hits and return the same ids and distances as the requests run alone
    (the shared threshold bounds the k-th distance from above, so no true
    neighbour is pruned); distinct queries are untouched."""
    cp, co, db = served_db
    reqs = _requests(15, 17)
    k = 10
    share = tsim.api.FLAG_SHARE_THRESHOLDS
    alone = [tsim.knn(cuda_ctx, db, qp, qo, m, k, stats=False, **PARAMS[m]) for m, qp, qo in reqs]
    with tsim.Server(cuda_ctx, db, slots=4, hbm_budget_bytes=512 << 20) as srv:
        first = [srv.wait(srv.submit(qp, qo, m, k, flags=share, **PARAMS[m])) for m, qp, qo in reqs]
        st1 = srv.stats()
        again = [srv.submit(qp, qo, m, k, flags=share, **PARAMS[m]) for m, qp, qo in reqs]
        second = [srv.wait(t) for t in again]
        st2 = srv.stats()
        # a query never seen before gets no shared threshold
        _, qn, on = _requests(1, 99)[0]
        srv.wait(srv.submit(qn, on, "dtw", k, flags=share, **PARAMS["dtw"]))
        st3 = srv.stats()
    nq = sum(len(qo) - 1 for _, _, qo in reqs)
    assert st1["shared_threshold_hits"] == 0
    assert st2["shared_threshold_hits"] == nq
    assert st3["shared_threshold_hits"] == nq
    for (m, qp, qo), (ia, da, _), (i1, d1, f1), (i2, d2, f2) in zip(reqs, alone, first, second):
        assert f1["status"] == 0 and f2["status"] == 0
        assert np.array_equal(ia, i1) and np.array_equal(ia, i2), m
        assert np.array_equal(da, d1) and np.array_equal(da, d2), m
