"""Host logic without a GPU: the seeded generators behind every workload
(shapes, distributions, determinism) and the serving load generator driven
through a fake server (pacing, latency accounting, summaries)."""
import threading
import time

import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G


def test_random_walks_shape_starts_and_steps():
    lens = G.uniform_lengths(400, 64, 512, 11)
    assert lens.min() >= 64 and lens.max() <= 512
    pts, off = G.random_walks(400, lens, 12)
    assert pts.dtype == np.float32 and pts.shape == (int(lens.sum()), 2)
    assert off[0] == 0 and np.array_equal(np.diff(off), lens)
    starts = pts[off[:-1]]
    assert starts.min() >= 0.0 and starts.max() < 100.0
    # steps inside trajectories: N(0, 1) per coordinate
    d = np.diff(pts.astype(np.float64), axis=0)
    inside = np.ones(len(d), bool)
    inside[off[1:-1] - 1] = False  # the jump from one trajectory's end to the next start
    d = d[inside]
    assert abs(d.mean()) < 0.02 and abs(d.std() - 1.0) < 0.02
    # seeded: the same call gives the same data, another seed other data
    pts2, off2 = G.random_walks(400, lens, 12)
    assert np.array_equal(pts, pts2) and np.array_equal(off, off2)
    assert not np.array_equal(pts, G.random_walks(400, lens, 13)[0])


def test_student_t_steps_have_heavy_tails():
    pn, on = G.random_walks(50, 2000, 5)
    pt, ot = G.random_walks(50, 2000, 5, step="student_t", nu=3.0)

    def kurt(pts, off):
        d = np.concatenate([np.diff(pts[off[i]:off[i + 1], 0].astype(np.float64))
                            for i in range(len(off) - 1)])
        d = d - d.mean()
        return (d ** 4).mean() / (d ** 2).mean() ** 2

    assert 2.8 < kurt(pn, on) < 3.2  # normal: 3
    assert kurt(pt, ot) > 6.0        # t with 3 degrees of freedom: heavy tails


def test_lognormal_lengths_clipped():
    lens = G.lognormal_lengths(20000, np.log(200), 0.6, 32, 1024, 3)
    assert lens.dtype == np.int64 and lens.min() == 32 and lens.max() == 1024
    assert 180 < np.median(lens) < 220


def test_reference_style_generators():
    num_t, n, m = 20, 64, 48
    t1 = G.ref_base_trajectories(num_t, n, 7)
    assert t1.shape == (num_t * n, 2) and t1.min() >= 0.0 and t1.max() <= 1000.0
    steps = np.abs(np.diff(t1.reshape(num_t, n, 2), axis=1))
    assert steps.max() <= 1.0 + 1e-3  # uniform steps in [-1, 1], clamped
    t2 = G.ref_similar_trajectories(t1, num_t, n, m, 2.0, 8)
    assert t2.shape == (num_t * m, 2)
    src = np.clip(np.rint(np.arange(m) * (n - 1) / (m - 1)).astype(int), 0, n - 1)
    base = t1.reshape(num_t, n, 2)[:, src]
    assert np.abs(t2.reshape(num_t, m, 2) - base).max() <= 2.0 + 1e-3


def test_device_random_walks_on_the_host():
    pytest.importorskip("torch")
    from cudaruntime1_gb300 import serving
    pts, off, ml = serving.device_random_walks(300, 50, 500, 21, device="cpu")
    lens = np.diff(off.numpy())
    assert lens.min() >= 50 and lens.max() <= 500 and ml == lens.max()
    p = pts.numpy()
    assert p.shape == (int(off[-1]), 2)
    assert p[off.numpy()[:-1]].min() >= 0.0 and p[off.numpy()[:-1]].max() < 100.0


class FakeServer:
    """submit/wait like cudaruntime1_gb300.api.Server: each request takes
    `service_ms` on one of `slots` workers, measured from its submission."""

    def __init__(self, service_ms=2.0, slots=4):
        self.service = service_ms / 1e3
        self.lock = threading.Lock()
        self.free_at = [0.0] * slots
        self.reqs = {}
        self.next = 1

    def submit(self, qp, qo, measure, k=10, **kw):
        now = time.perf_counter()
        with self.lock:
            i = int(np.argmin(self.free_at))
            start = max(now, self.free_at[i])
            done = start + self.service
            self.free_at[i] = done
            t = self.next
            self.next += 1
            self.reqs[t] = (now, start, done, len(qo) - 1, k)
        return t

    def wait(self, ticket, timeout_ms=-1):
        with self.lock:
            sub, start, done, nq, k = self.reqs.pop(ticket)
        delay = done - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        info = {"status": 0, "nq": nq, "k": k, "queue_ms": (start - sub) * 1e3,
                "latency_ms": (done - sub) * 1e3, "device_ms": self.service * 1e3,
                "scratch_bytes": 0, "inflight_at_admit": 0}
        return np.zeros((nq, k), np.int32), np.zeros((nq, k), np.float32), info


def test_open_loop_paces_arrivals_and_accounts_latency():
    from cudaruntime1_gb300 import serving
    reqs = serving.make_requests(200, 16, 64, 4)
    assert {m for m, _, _ in reqs} <= set(serving.MEASURE_PARAMS)
    assert all(16 <= int(qo[-1]) <= 64 for _, _, qo in reqs)
    srv = FakeServer(service_ms=2.0, slots=4)
    out = serving.run_open_loop(srv, reqs, rate=1000.0, seed=1)
    assert out["requests"] == 200 and out["offered_rps"] == 1000.0
    # 200 arrivals at 1000/s take about 0.2 s; the server keeps up
    assert 600.0 < out["achieved_rps"] < 1300.0
    assert out["p50_ms"] >= 2.0 and out["p50_ms"] < 20.0
    assert out["p99_ms"] >= out["p50_ms"]
    assert sum(v["requests"] for v in out["per_measure"].values()) == 200


def test_closed_loop_measures_capacity():
    from cudaruntime1_gb300 import serving
    reqs = serving.make_requests(64, 16, 32, 5, measures=["dtw", "lcss"])
    assert {m for m, _, _ in reqs} == {"dtw", "lcss"}
    srv = FakeServer(service_ms=5.0, slots=4)
    out = serving.run_closed_loop(srv, reqs)
    # 64 requests x 5 ms on 4 slots: 80 ms, capacity about 800 requests/s
    assert 500.0 < out["achieved_rps"] < 850.0
    # all queued at once: later requests wait for earlier ones
    assert out["queue_p99_ms"] > 50.0 and out["queue_p50_ms"] > 20.0
    assert set(out["per_measure"]) == {"dtw", "lcss"}
