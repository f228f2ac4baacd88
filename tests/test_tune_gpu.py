"""Autotuner (tsim_autotune): it times the launch choices on a request and
records the fastest per shape class; results never depend on the choices,
and the table survives a save / load round trip."""
import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu


def _device_request(qp, qo):
    import torch
    return (torch.from_numpy(qp).cuda(), torch.from_numpy(np.asarray(qo, np.int64)).cuda(),
            len(qo) - 1, int(np.max(np.diff(qo))))


@pytest.mark.parametrize("measure,kw", [("dtw", dict(band_pct=10)), ("lcss", dict(epsilon=0.5, delta=8)),
                                        ("frechet", dict()), ("hausdorff", dict())])
def test_autotune_keeps_results_and_round_trips(tsim, tmp_path, measure, kw):
    import torch
    ctx = tsim.Context(0)
    cp, co = G.random_walks(2000, G.uniform_lengths(2000, 16, 160, 3), 4)
    qp, qo = G.random_walks(40, G.uniform_lengths(40, 16, 160, 5), 6)
    db = tsim.Database(ctx, cp, co)
    ids0, d0, _ = tsim.knn(ctx, db, qp, qo, measure, 10, stats=False, **kw)
    qpt, qot, nq, maxq = _device_request(qp, qo)
    torch.cuda.synchronize()
    r = ctx.autotune(db, qpt.data_ptr(), qot.data_ptr(), nq, maxq, measure, 10, reps=3, **kw)
    assert r["tried"] >= 1 and r["best_ms"] > 0 and r["default_ms"] > 0
    assert r["streams"] in (1, 2, 4, 8)
    assert ctx.tuning_count() == 1
    # a tuned request (eager and through graph replay) gives the same answer
    for _ in range(3):
        ids1, d1, _ = tsim.knn(ctx, db, qp, qo, measure, 10, stats=False, **kw)
        assert np.array_equal(ids0, ids1) and np.array_equal(d0, d1)
    path = tmp_path / "tuning.txt"
    ctx.save_tuning(path)
    ctx.clear_tuning()
    assert ctx.tuning_count() == 0
    ctx.load_tuning(path)
    assert ctx.tuning_count() == 1
    ids2, d2, _ = tsim.knn(ctx, db, qp, qo, measure, 10, stats=False, **kw)
    assert np.array_equal(ids0, ids2) and np.array_equal(d0, d2)
    # a table tuned on another device is refused
    bad = tmp_path / "other.txt"
    bad.write_text(path.read_text().replace("# tsim tuning v1 ", "# tsim tuning v1 X", 1))
    with pytest.raises(tsim.api._lib.TsimError):
        ctx.load_tuning(bad)
    db.close()
    ctx.close()

