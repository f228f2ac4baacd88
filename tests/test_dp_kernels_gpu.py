"""The DP kernels pair by pair against the FP64 oracle: every precision
(FP32, compensated FP32, FP64) on every kernel (round-striped; anti-diagonal
with a warp, two warps or a CTA per pair; a lane per pair; band-relative
with a warp per pair), across
query/candidate shapes, bands and windows.
FP64 values must be bit-identical, compensated within 1e-9, FP32 within the
FP32 error bound (n+m+8)*2^-24, LCSS counts exact."""
import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G

pytestmark = pytest.mark.gpu


def _setup(nq, nc, lo, hi, seed):
    import torch
    ql = G.uniform_lengths(nq, lo, hi, seed)
    cl = G.uniform_lengths(nc, lo, hi, seed + 1)
    qp, qo = G.random_walks(nq, ql, seed + 2)
    cp, co = G.random_walks(nc, cl, seed + 3)
    # nearby pairs too: candidates 0..nq-1 are noisy copies of the queries, resampled
    for i in range(min(nq, nc)):
        src = np.linspace(0, ql[i] - 1, cl[i]).round().astype(int)
        cp[co[i]:co[i + 1]] = qp[qo[i] + src] + 0.3 * np.random.default_rng(i).standard_normal((cl[i], 2)).astype(np.float32)
    rng = np.random.default_rng(seed + 4)
    pairs = np.stack([rng.integers(0, nq, 600), rng.integers(0, nc, 600)], 1).astype(np.int32)
    pairs[:nq, 0] = np.arange(nq)
    pairs[:nq, 1] = np.arange(nq)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
           dict(qp=qp, qo=qo, cp=cp, co=co, pr=pairs).items()}
    return qp, qo, cp, co, pairs, dev, int(ql.max()), int(cl.max())


CASES = [
    ("dtw", dict(band_pct=10, cost=0), 16, 120),
    ("dtw", dict(band_pct=10, cost=0), 64, 512),
    ("dtw", dict(band_pct=30, cost=1), 8, 60),
    ("dtw", dict(band_pct=-1, cost=0), 2, 40),
    ("frechet", dict(), 2, 30),
    ("frechet", dict(), 20, 90),
    ("lcss", dict(epsilon=1.0, delta=5), 10, 150),
    ("lcss", dict(epsilon=0.5, delta=-1), 2, 28),
    # full rows past 31*4+1 columns: anti-diagonal passes with R = 8 and 16
    ("dtw", dict(band_pct=-1, cost=0), 130, 480),
    ("frechet", dict(), 130, 240),
    ("lcss", dict(epsilon=0.5, delta=200), 130, 300),
]


@pytest.mark.parametrize("measure,kw,lo,hi", CASES)
def test_dp_pairs_all_kernels(tsim, cuda_ctx, oracle, measure, kw, lo, hi):
    import torch
    from cudaruntime1_gb300 import api
    qp, qo, cp, co, pairs, dev, mq, mc = _setup(12, 80, lo, hi, 31 + lo + hi)
    okw = dict(kw)
    if "epsilon" in okw:
        okw["eps"] = okw.pop("epsilon")
    want = np.array([oracle.pair(measure, qp[qo[a]:qo[a + 1]], cp[co[b]:co[b + 1]], **okw)
                     for a, b in pairs])
    n_ = np.diff(qo)[pairs[:, 0]]
    m_ = np.diff(co)[pairs[:, 1]]
    fp32 = {}
    for kernel in (1, 2, 3, 4, 5, 6):
        for precision in ((0,) if measure == "lcss" else (0, 1, 2)):
            o32 = torch.full((len(pairs),), float("nan"), dtype=torch.float32, device="cuda")
            o64 = torch.full((len(pairs),), float("nan"), dtype=torch.float64, device="cuda")
            ctx = cuda_ctx
            api.dp_pairs(ctx, measure, precision, kernel, dev["qp"].data_ptr(), dev["qo"].data_ptr(),
                         mq, dev["cp"].data_ptr(), dev["co"].data_ptr(), mc, dev["pr"].data_ptr(),
                         len(pairs), o32.data_ptr(), o64.data_ptr(), **kw)
            torch.cuda.synchronize()
            got = (o32 if precision == 0 else o64).cpu().numpy().astype(np.float64)
            if precision == 0:
                fp32[kernel] = o32.cpu().numpy()
            w = want ** 2 if measure == "frechet" else want  # kernels report Frechet squared
            tag = (measure, kernel, precision)
            assert np.array_equal(np.isfinite(got), np.isfinite(w)), tag
            f = np.isfinite(w)
            if measure == "lcss":
                assert np.array_equal(got, w), tag
                continue
            rel = np.abs(got[f] - w[f]) / np.maximum(w[f], 1e-30)
            if precision == 2:
                ok = np.array_equal(got[f], w[f]) if measure != "frechet" else rel.max() <= 1e-15
                assert ok, (tag, rel.max())
            elif precision == 1:  # DTW: 4u from the FP32 costs; Frechet: double-float
                lim = 4.5 * 2.0 ** -24 if measure == "dtw" else 1e-9
                assert rel.max() <= lim, (tag, rel.max(), np.argmax(rel), pairs[f][np.argmax(rel)])
            else:
                bound = (n_[f] + m_[f] + 8) * 2.0 ** -24 * 1.01 + 1e-12
                assert np.all(rel <= bound), (tag, rel.max(), np.argmax(rel / bound))
    # the same cells with the same operations: FP32 values agree to the bit
    # between the warp-per-pair, lane-per-pair and band-relative kernels
    for kernel in (5, 6):
        assert np.array_equal(fp32[2].view(np.uint32), fp32[kernel].view(np.uint32)), \
            (measure, kernel)
