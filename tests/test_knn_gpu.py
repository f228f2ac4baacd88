"""Exact kNN on the GPU against the FP64 brute-force oracle: ids bit-exact
(ties by candidate index), FP64 distances bit-identical, float distances
within 1e-5 relative (they are the FP64 values rounded once)."""
import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu
REL_TOL = 1e-5


def _db(nc, lo, hi, seed, step="normal"):
    lens = G.uniform_lengths(nc, lo, hi, seed)
    return G.random_walks(nc, lens, seed + 1, step=step)


def _device_knn(tsim, ctx, db, qp, qo, measure, k, **kw):
    import torch
    qpt = torch.from_numpy(qp).cuda()
    qot = torch.from_numpy(np.asarray(qo, np.int64)).cuda()
    nq = len(qo) - 1
    ids = torch.empty(nq * k, dtype=torch.int32, device="cuda")
    d = torch.empty(nq * k, dtype=torch.float32, device="cuda")
    d64 = torch.empty(nq * k, dtype=torch.float64, device="cuda")
    maxq = int(np.max(np.diff(qo)))
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    st = tsim.knn_device(ctx, db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, ids.data_ptr(),
                         d.data_ptr(), d64.data_ptr(), measure, k, stats=True, **kw)
    torch.cuda.synchronize()
    return (ids.cpu().numpy().reshape(nq, k), d.cpu().numpy().reshape(nq, k),
            d64.cpu().numpy().reshape(nq, k), st)


CASES = [
    ("dtw", dict(band_pct=10, cost=0)),
    ("dtw", dict(band_pct=-1, cost=0)),
    ("dtw", dict(band_pct=20, cost=1)),
    ("lcss", dict(epsilon=0.5, delta=5)),
    ("lcss", dict(epsilon=0.25, delta=-1)),
    ("frechet", dict()),
    ("hausdorff", dict()),
]


@pytest.mark.parametrize("pruned", [False, True])
@pytest.mark.parametrize("measure,kw", CASES)
def test_knn_matches_fp64_oracle(tsim, cuda_ctx, oracle, measure, kw, pruned):
    cp, co = _db(700, 16, 120, 100)
    ql = G.uniform_lengths(9, 16, 120, 7)
    qp, qo = G.random_walks(9, ql, 8)
    k = 10
    db = tsim.Database(cuda_ctx, cp, co)
    okw = dict(kw)
    if "epsilon" in okw:
        okw["eps"] = okw.pop("epsilon")
    want_ids, want_d = oracle.knn(measure, qp, qo, cp, co, k, **okw)
    if pruned:  # the bound stages, which a request this small skips by default
        kw = dict(kw, flags=tsim.api.FLAG_ALWAYS_PRUNE)
    ids, d, d64, st = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, k, **kw)
    assert np.array_equal(ids, want_ids), (ids, want_ids)
    if measure == "lcss":
        assert np.array_equal(d.astype(np.float64), want_d)
    else:
        fin = np.isfinite(want_d)
        assert np.array_equal(np.isfinite(d64), fin)
        rel = np.abs(d.astype(np.float64)[fin] - want_d[fin]) / np.maximum(want_d[fin], 1e-30)
        assert rel.max() <= REL_TOL
        # DTW's compensated re-score (FP32 costs within 4 2^-24, path sum
        # compensated) and the other measures' FP32 values (FP64 only for
        # near-ties) are all within a few 2^-24 of FP64
        rel64 = np.abs(d64[fin] - want_d[fin]) / np.maximum(want_d[fin], 1e-30)
        assert rel64.max() <= 1e-6, rel64.max()
        # forced FP64 re-score: bit-identical to the FP64 oracle
        kw64 = dict(kw, flags=kw.get("flags", 0) | tsim.api.FLAG_FP64_RESCORE)
        ids2, _, d64b, st2 = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, k, **kw64)
        assert np.array_equal(ids2, want_ids)
        assert np.array_equal(d64b, want_d)
        assert st2["rescored_fp64"] >= np.isfinite(want_d).sum()
    # the host-pointer entry point gives the same answer
    ids_h, d_h, _ = tsim.knn(cuda_ctx, db, qp, qo, measure, k, **kw)
    assert np.array_equal(ids_h, ids) and np.array_equal(d_h, d)
    db.close()


def test_knn_edge_cases(tsim, cuda_ctx, oracle):
    # fewer candidates than k; single-point trajectories; duplicates (ties)
    cp, co = _db(5, 1, 6, 300)
    qp, qo = G.random_walks(3, [1, 4, 6], 301)
    db = tsim.Database(cuda_ctx, cp, co)
    for measure, kw, okw in [("dtw", dict(band_pct=10), dict(band_pct=10)),
                             ("frechet", {}, {}),
                             ("lcss", dict(epsilon=30.0, delta=2), dict(eps=30.0, delta=2))]:
        want_ids, want_d = oracle.knn(measure, qp, qo, cp, co, 8, **okw)
        ids, d, d64, _ = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 8, **kw)
        assert np.array_equal(ids, want_ids), (measure, ids, want_ids)
    db.close()
    # exact duplicates in the database: ties broken by index
    base, bo = G.random_walks(4, 30, 400)
    cp = np.concatenate([base, base[bo[1]:bo[2]], base[bo[1]:bo[2]]])
    co = np.concatenate([bo, [bo[-1] + 30, bo[-1] + 60]])
    db = tsim.Database(cuda_ctx, cp, co)
    qp = base[bo[1]:bo[2]].copy()
    qo = np.array([0, 30])
    for measure in ("dtw", "frechet", "lcss"):
        want_ids, _ = oracle.knn(measure, qp, qo, cp, co, 6)
        ids, _, _, _ = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 6)
        assert np.array_equal(ids, want_ids), (measure, ids, want_ids)
        assert list(ids[0][:3]) == [1, 4, 5]
    db.close()


def test_knn_longer_queries_than_candidates(tsim, cuda_ctx, oracle):
    cp, co = _db(300, 10, 40, 500)
    qp, qo = G.random_walks(4, [200, 150, 90, 300], 501)
    db = tsim.Database(cuda_ctx, cp, co)
    for measure, kw, okw in [("dtw", dict(band_pct=30), dict(band_pct=30)),
                             ("lcss", dict(epsilon=1.0, delta=4), dict(eps=1.0, delta=4))]:
        want_ids, want_d = oracle.knn(measure, qp, qo, cp, co, 5, **okw)
        ids, d, d64, _ = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 5, **kw)
        assert np.array_equal(ids, want_ids), measure
    db.close()


def test_context_destroyed_before_database(tsim):
    """Destroying a context releases its databases' device memory and
    detaches them; closing such a database afterwards is safe and using it is
    an error, whatever order Python collects the objects in."""
    ctx = tsim.Context(0)
    cp, co = _db(50, 8, 20, 700)
    db = tsim.Database(ctx, cp, co)
    qp, qo = G.random_walks(1, 10, 701)
    ids, _, _ = tsim.knn(ctx, db, qp, qo, "dtw", 3)
    ctx2 = tsim.Context(0)
    with pytest.raises(tsim._lib.TsimError):
        tsim.knn(ctx2, db, qp, qo, "dtw", 3)  # wrong context
    ctx.close()
    db.close()
    ctx2.close()


def test_host_calls_two_contexts_growing_requests(tsim, oracle):
    """Host-pointer kNN on two contexts of one thread, interleaved, with
    requests that grow (each context's device staging is its own and grows
    with the request); a NULL point array is an argument error."""
    import ctypes as C
    cp, co = _db(200, 8, 40, 720)
    ctxs = [tsim.Context(0), tsim.Context(0)]
    dbs = [tsim.Database(c, cp, co) for c in ctxs]
    for i, nq in enumerate([1, 3, 40, 2, 90]):
        qp, qo = G.random_walks(nq, G.uniform_lengths(nq, 4, 60, 730 + i), 740 + i)
        want_ids, _ = oracle.knn("dtw", qp, qo, cp, co, 4, band_pct=20)
        for c, db in zip(ctxs, dbs):
            ids, _, _ = tsim.knn(c, db, qp, qo, "dtw", 4, band_pct=20)
            assert np.array_equal(ids, want_ids), (nq, ids, want_ids)
    h = C.c_void_p()
    off = np.array([0, 3], np.int64)
    st = ctxs[0].L.tsim_db_create(ctxs[0].h, None, off.ctypes.data, 1, C.byref(h))
    assert st == tsim._lib.TSIM_ERR_INVALID_ARG and not h.value
    for db in dbs:
        db.close()
    for c in ctxs:
        c.close()


def test_euclidean_knn_prefix_rule_and_long_pairs(tsim, cuda_ctx, oracle):
    """Lock-step Euclidean: candidates of length 64 and a few of 1,100 points
    (> 1024: the FP64 accumulation branch) against queries of 1,100 points;
    a candidate is compared with the query's first m points."""
    rng = np.random.default_rng(9)
    lens = np.where(rng.random(600) < 0.02, 1100, 64)
    lens[:3] = 1100
    cp, co = G.random_walks(600, lens, 901, step="student_t")
    qp, qo = G.random_walks(5, 1100, 902, step="student_t")
    # plant near matches: candidate 1 = query 0 plus noise, candidate 7 = query 1 prefix
    cp[co[1]:co[2]] = qp[qo[0]:qo[0] + 1100] + 0.01
    cp[co[7]:co[8]] = qp[qo[1]:qo[1] + lens[7]] + 0.02
    db = tsim.Database(cuda_ctx, cp, co)
    want_ids, want_d = oracle.knn("euclidean", qp, qo, cp, co, 10)
    ids, d, d64, st = _device_knn(tsim, cuda_ctx, db, qp, qo, "euclidean", 10)
    assert np.array_equal(ids, want_ids)
    assert ids[0][0] == 1 and ids[1][0] == 7
    fin = np.isfinite(want_d)
    assert np.max(np.abs(d[fin] - want_d[fin]) / want_d[fin]) <= REL_TOL
    ids2, _, d64b, _ = _device_knn(tsim, cuda_ctx, db, qp, qo, "euclidean", 10,
                                   flags=tsim.api.FLAG_FP64_RESCORE)
    assert np.array_equal(ids2, want_ids) and np.array_equal(d64b, want_d)
    db.close()


def test_query_batches(tsim, cuda_ctx, oracle):
    """More query x candidate pairs than one batch holds: the queries are
    processed in slices with the same results."""
    cp, co = _db(70000, 8, 24, 950)
    qp, qo = G.random_walks(300, G.uniform_lengths(300, 8, 24, 951), 952)
    db = tsim.Database(cuda_ctx, cp, co)
    sel = [0, 137, 299]
    ids, d, d64, _ = _device_knn(tsim, cuda_ctx, db, qp, qo, "frechet", 4)
    for q in sel:
        sub_o = np.array([0, qo[q + 1] - qo[q]])
        wi, wd = oracle.knn("frechet", qp[qo[q]:qo[q + 1]], sub_o, cp, co, 4)
        assert np.array_equal(ids[q], wi[0]), q
    db.close()


@pytest.mark.parametrize("measure,kw", [("dtw", dict(band_pct=10)), ("lcss", dict(epsilon=0.5, delta=5)),
                                        ("hausdorff", {})])
def test_pruning_never_changes_the_answer(tsim, cuda_ctx, measure, kw):
    """TSIM_FLAG_NO_PRUNE refines every pair; the pruned pipeline must return
    the same ids and distances."""
    cp, co = _db(1500, 20, 90, 1200)
    qp, qo = G.random_walks(6, G.uniform_lengths(6, 20, 90, 1201), 1202)
    db = tsim.Database(cuda_ctx, cp, co)
    ids, d, _, st = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 10,
                                flags=tsim.api.FLAG_ALWAYS_PRUNE, **kw)
    ids2, d2, _, st2 = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 10,
                                   flags=tsim.api.FLAG_NO_PRUNE, **kw)
    assert np.array_equal(ids, ids2) and np.array_equal(d, d2)
    assert st2["pairs_refined"] >= 6 * 1500 and st["pairs_refined"] < st2["pairs_refined"]
    db.close()


def test_graph_replay_follows_inputs(tsim, cuda_ctx, oracle):
    """Repeated requests of one shape replay a captured CUDA graph; the graph
    re-reads its input buffers, so changed query points give the new answer."""
    import torch
    cp, co = _db(900, 20, 60, 1300)
    qp, qo = G.random_walks(24, G.uniform_lengths(24, 20, 60, 1301), 1302)
    db = tsim.Database(cuda_ctx, cp, co)
    stream = torch.cuda.Stream()
    cuda_ctx.set_stream(stream.cuda_stream)
    qpt = torch.from_numpy(qp).cuda()
    qot = torch.from_numpy(qo).cuda()
    k = 5
    ids = torch.empty(24 * k, dtype=torch.int32, device="cuda")
    d = torch.empty(24 * k, dtype=torch.float32, device="cuda")
    want, _ = oracle.knn("dtw", qp, qo, cp, co, k, band_pct=10)
    cuda_ctx.counters(reset=True)
    for it in range(4):  # eager, capture, replay, replay
        tsim.knn_device(cuda_ctx, db, qpt.data_ptr(), qot.data_ptr(), 24, 60, ids.data_ptr(),
                        d.data_ptr(), None, "dtw", k, band_pct=10)
        stream.synchronize()
        assert np.array_equal(ids.cpu().numpy().reshape(24, k), want), it
    launches = cuda_ctx.counters(reset=True)["launches"]
    assert launches > 0
    qp2 = qp[::-1].copy()  # new query points in the same buffer
    qpt.copy_(torch.from_numpy(qp2))
    stream.synchronize()
    tsim.knn_device(cuda_ctx, db, qpt.data_ptr(), qot.data_ptr(), 24, 60, ids.data_ptr(),
                    d.data_ptr(), None, "dtw", k, band_pct=10)
    stream.synchronize()
    want2, _ = oracle.knn("dtw", qp2, qo, cp, co, k, band_pct=10)
    assert np.array_equal(ids.cpu().numpy().reshape(24, k), want2)
    cuda_ctx.set_stream(None)
    db.close()


@pytest.mark.parametrize("measure,kw", [("dtw", dict(band_pct=-1, cost=0)), ("frechet", dict())])
def test_knn_full_rows_long_candidates(tsim, cuda_ctx, oracle, measure, kw):
    """Full-row DP of candidates longer than 31*4+1 points: anti-diagonal
    passes with 8 and 16 rows per lane-group, with early abandon."""
    cp, co = _db(600, 130, 480, 300)
    ql = G.uniform_lengths(6, 130, 480, 301)
    qp, qo = G.random_walks(6, ql, 302)
    db = tsim.Database(cuda_ctx, cp, co)
    want_ids, want_d = oracle.knn(measure, qp, qo, cp, co, 10, **kw)
    ids, d, d64, st = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 10, **kw)
    assert np.array_equal(ids, want_ids)
    rel = np.abs(d.astype(np.float64) - want_d) / np.maximum(want_d, 1e-30)
    assert rel.max() <= REL_TOL
    db.close()


@pytest.mark.parametrize("measure,kw", [("dtw", dict(band_pct=10)), ("lcss", dict(epsilon=0.5, delta=20))])
def test_knn_mixed_query_lengths_one_call(tsim, cuda_ctx, oracle, measure, kw):
    """Queries of 512, 600 and 1,100 points in one call: their sparse tables
    share a stride sized for the longest, although a 512-row table is larger
    than a 600-row one (rows are grouped in blocks beyond 512)."""
    cp, co = _db(1500, 40, 200, 400)
    qp, qo = G.random_walks(4, [512, 600, 300, 1100], 401)
    db = tsim.Database(cuda_ctx, cp, co)
    okw = dict(kw)
    if "epsilon" in okw:
        okw["eps"] = okw.pop("epsilon")
    want_ids, want_d = oracle.knn(measure, qp, qo, cp, co, 10, **okw)
    ids, d, _, _ = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 10,
                               flags=tsim.api.FLAG_ALWAYS_PRUNE, **kw)
    assert np.array_equal(ids, want_ids)
    db.close()


@pytest.mark.parametrize("pruned", [False, True])
def test_knn_k64_with_many_ties(tsim, cuda_ctx, oracle, pruned):
    """k at its maximum (64) over a database in which every trajectory occurs
    eight times: the block selections (radix passes over the packed keys,
    ties broken by candidate index) against the oracle."""
    base, bo = _db(60, 12, 70, 900)
    reps = 8
    parts, offs = [], [0]
    for r in range(reps):
        for t in range(60):
            seg = base[bo[t]:bo[t + 1]]
            parts.append(seg)
            offs.append(offs[-1] + len(seg))
    cp = np.concatenate(parts)
    co = np.array(offs, np.int64)
    ql = G.uniform_lengths(6, 12, 70, 901)
    qp, qo = G.random_walks(6, ql, 902)
    db = tsim.Database(cuda_ctx, cp, co)
    k = 64
    for measure, kw, okw in [("dtw", dict(band_pct=20), dict(band_pct=20)),
                             ("lcss", dict(epsilon=1.5, delta=-1), dict(eps=1.5, delta=-1)),
                             ("hausdorff", {}, {})]:
        want_ids, want_d = oracle.knn(measure, qp, qo, cp, co, k, **okw)
        if pruned:
            kw = dict(kw, flags=tsim.api.FLAG_ALWAYS_PRUNE)
        ids, d, _, _ = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, k, **kw)
        assert np.array_equal(ids, want_ids), (measure, pruned)
    db.close()


def test_frechet_fp64_window_and_tiny_values(tsim, cuda_ctx, oracle):
    """The exact FP64 Frechet re-score (FP64 costs only in the window around
    the FP32 optimum) against the oracle, bit for bit: exact duplicates (value
    0), near-duplicates whose optimum is below 1e-20 (every cell in FP64) and
    offsets that keep it in the window."""
    base, bo = G.random_walks(6, 40, 1200)
    parts, offs = [], [0]
    rng = np.random.default_rng(1201)
    for t in range(6):
        seg = base[bo[t]:bo[t + 1]].astype(np.float64)
        for scale in (0.0, 1e-12, 1e-3, 0.5):
            v = seg + scale * rng.standard_normal(seg.shape)
            parts.append(v.astype(np.float32))
            offs.append(offs[-1] + len(seg))
    cp = np.concatenate(parts)
    co = np.array(offs, np.int64)
    qp = np.concatenate([base[bo[t]:bo[t + 1]] for t in (0, 3)])
    qo = np.array([0, 40, 80], np.int64)
    db = tsim.Database(cuda_ctx, cp, co)
    k = 8
    want_ids, want_d = oracle.knn("frechet", qp, qo, cp, co, k)
    for flags in (tsim.api.FLAG_FP64_RESCORE,
                  tsim.api.FLAG_FP64_RESCORE | tsim.api.FLAG_ALWAYS_PRUNE):
        ids, _, d64, _ = _device_knn(tsim, cuda_ctx, db, qp, qo, "frechet", k, flags=flags)
        assert np.array_equal(ids, want_ids)
        assert np.array_equal(d64, want_d)
    db.close()


@pytest.mark.parametrize("pruned", [False, True])
def test_plain_small_workload_full_size(tsim, cuda_ctx, oracle, pruned):
    """The small plain workload at its own size: 8 queries x 1,024 candidates,
    every trajectory 128 points (N(0,1) random walks), all five measures with
    the full DP (no band, no LCSS window), top-10 -- ids bit-exact against
    the FP64 brute-force oracle, LCSS counts exact, distances within 1e-5."""
    from cudaruntime1_gb300 import datagen as G
    cp, co = G.random_walks(1024, 128, 11 + 3)
    qp, qo = G.random_walks(8, 128, 11 + 4)
    db = tsim.Database(cuda_ctx, cp, co)
    runs = [("dtw", dict(band_pct=-1, cost=0)), ("lcss", dict(epsilon=0.5, delta=-1)),
            ("frechet", {}), ("hausdorff", {}), ("euclidean", {})]
    for measure, kw in runs:
        okw = dict(kw)
        if "epsilon" in okw:
            okw["eps"] = okw.pop("epsilon")
        want_ids, want_d = oracle.knn(measure, qp, qo, cp, co, 10, **okw)
        if pruned:
            kw = dict(kw, flags=tsim.api.FLAG_ALWAYS_PRUNE)
        ids, d, d64, st = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 10, **kw)
        assert np.array_equal(ids, want_ids), measure
        if measure == "lcss":
            assert np.array_equal(d.astype(np.float64), want_d)
        else:
            rel = np.abs(d.astype(np.float64) - want_d) / np.maximum(want_d, 1e-30)
            assert rel.max() <= REL_TOL, (measure, rel.max())
        assert st["pairs"] == 8 * 1024
    db.close()


@pytest.mark.parametrize("measure,kw", [("dtw", dict(band_pct=10, cost=0)),
                                        ("dtw", dict(band_pct=-1, cost=1)),
                                        ("lcss", dict(epsilon=0.5, delta=8)),
                                        ("frechet", {})])
def test_dp_kernel_choices_agree(tsim, cuda_ctx, oracle, measure, kw):
    """Rounds of many pairs run a lane per pair (dp_lane.cu), DTW and Frechet
    rounds start on the band-relative kernel (dp_wave.cu); with
    TSIM_FLAG_NO_LANE_DP / TSIM_FLAG_NO_WAVE_DP they run on the row-group
    kernels instead.  Every choice gives the same ids and distance bits,
    brute force (36,000 pairs, past the lane kernel's gate) and pruned, and
    the ids equal the FP64 oracle's."""
    cp, co = _db(3000, 16, 300, 91)
    ql = G.uniform_lengths(12, 16, 300, 92)
    qp, qo = G.random_walks(12, ql, 93)
    db = tsim.Database(cuda_ctx, cp, co)
    okw = {("eps" if k == "epsilon" else k): v for k, v in kw.items()}
    want_ids, _ = oracle.knn(measure, qp, qo, cp, co, 10, **okw)
    off = tsim.api.FLAG_NO_LANE_DP | tsim.api.FLAG_NO_WAVE_DP
    for extra in (0, tsim.api.FLAG_ALWAYS_PRUNE):
        base = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 10, flags=extra | off, **kw)
        assert np.array_equal(base[0], want_ids), (measure, extra)
        for choice in (0, tsim.api.FLAG_NO_LANE_DP, tsim.api.FLAG_NO_WAVE_DP):
            got = _device_knn(tsim, cuda_ctx, db, qp, qo, measure, 10, flags=extra | choice, **kw)
            assert np.array_equal(got[0], base[0]), (measure, extra, choice)
            assert np.array_equal(got[1].view(np.uint32), base[1].view(np.uint32)), \
                (measure, extra, choice)
            if measure != "lcss":  # the FP64 re-scored distances
                assert np.array_equal(got[2].view(np.uint64), base[2].view(np.uint64)), \
                    (measure, extra, choice)
    db.close()
