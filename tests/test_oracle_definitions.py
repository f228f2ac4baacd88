"""The FP64 oracle against a second, independent restatement of the five
measures on tiny inputs: DTW and discrete Frechet as the minimum over every
enumerated warping path (the band written as the predicate
|i(m-1) - j(n-1)| <= w (min(n,m)-1), not as integer ramps), LCSS as the best
chain of matches chosen one next match at a time, Hausdorff and lock-step
Euclidean straight from their definitions.  Same FP64 operations per path, so
the values must be bit-identical."""
import math
from functools import lru_cache

import numpy as np
import pytest

from cudaruntime1_gb300 import datagen as G


def _d2(p, q):
    dx = float(p[0]) - float(q[0])
    dy = float(p[1]) - float(q[1])
    return dx * dx + dy * dy


def _band_w(n, m, pct):
    return -1 if pct < 0 else -(-pct * max(n, m) // 100)


def _in_band(i, j, n, m, w):
    if w < 0 or n <= 1:
        return True
    return abs(i * (m - 1) - j * (n - 1)) <= w * (min(n, m) - 1)


def _paths(n, m):
    """Every warping path from (0, 0) to (n-1, m-1), steps (1,0), (0,1), (1,1)."""
    out = []

    def walk(i, j, path):
        if i == n - 1 and j == m - 1:
            out.append(path)
            return
        for di, dj in ((1, 0), (0, 1), (1, 1)):
            if i + di < n and j + dj < m:
                walk(i + di, j + dj, path + [(i + di, j + dj)])

    walk(0, 0, [(0, 0)])
    return out


def dtw_paths(a, b, pct, euclid):
    n, m = len(a), len(b)
    w = _band_w(n, m, pct)
    best = math.inf
    for path in _paths(n, m):
        if not all(_in_band(i, j, n, m, w) for i, j in path):
            continue
        s = 0.0
        for i, j in path:  # the DP's order: cost + sum of the path so far
            c = _d2(a[i], b[j])
            s = (math.sqrt(c) if euclid else c) + s
        best = min(best, s)
    return best


def frechet_paths(a, b):
    return math.sqrt(min(max(_d2(a[i], b[j]) for i, j in path) for path in _paths(len(a), len(b))))


def lcss_next_match(a, b, eps, delta):
    n, m = len(a), len(b)
    f32 = np.float32

    def match(i, j):
        if delta >= 0 and abs(i - j) > delta:
            return False
        dx = abs(f32(a[i][0]) - f32(b[j][0]))  # FP32 differences, strict compare
        dy = abs(f32(a[i][1]) - f32(b[j][1]))
        return bool(dx < f32(eps) and dy < f32(eps))

    @lru_cache(maxsize=None)
    def best(i0, j0):
        r = 0
        for i in range(i0, n):
            for j in range(j0, m):
                if match(i, j):
                    r = max(r, 1 + best(i + 1, j + 1))
        return r

    return best(0, 0)


def hausdorff_def(a, b):
    def directed(x, y):
        return max(min(_d2(p, q) for q in y) for p in x)

    return math.sqrt(max(directed(a, b), directed(b, a)))


def euclid_def(q, c):
    if len(q) < len(c):
        return math.inf
    s = 0.0
    for i in range(len(c)):
        s += _d2(q[i], c[i])
    return math.sqrt(s)


def _cases(count, seed, hi=6):
    rng = np.random.default_rng(seed)
    for t in range(count):
        n, m = int(rng.integers(1, hi + 1)), int(rng.integers(1, hi + 1))
        pts, off = G.random_walks(2, [n, m], seed * 1000 + t, start_range=3.0)
        yield pts[off[0]:off[1]], pts[off[1]:off[2]]


@pytest.mark.parametrize("pct,cost", [(-1, 0), (-1, 1), (10, 0), (30, 0), (50, 1)])
def test_dtw_is_the_best_band_path(oracle, pct, cost):
    for a, b in _cases(40, 1 + pct % 7 + cost):
        want = dtw_paths(a, b, pct, euclid=(cost == oracle.COST_EUCLID))
        got = oracle.pair("dtw", a, b, band_pct=pct, cost=cost)
        assert got == want, (len(a), len(b), pct, cost, got, want)


def test_frechet_is_the_best_path_maximum(oracle):
    for a, b in _cases(40, 2):
        assert oracle.pair("frechet", a, b) == frechet_paths(a, b)


@pytest.mark.parametrize("eps,delta", [(0.5, -1), (1.0, 1), (2.0, 0), (0.25, 3)])
def test_lcss_is_the_longest_match_chain(oracle, eps, delta):
    rng = np.random.default_rng(30)
    counts = []
    for a, b in _cases(40, 3):
        # and a noisy copy of a with points dropped: long chains of matches
        keep = rng.random(len(a)) < 0.8
        near = (a[keep] + rng.normal(0.0, 0.2, (int(keep.sum()), 2))).astype(np.float32)
        for x, y in ((a, b), (a, near)):
            if len(y) == 0:
                continue
            want = lcss_next_match(x, y, eps, delta)
            assert oracle.pair("lcss", x, y, eps=eps, delta=delta) == want
            counts.append(want)
    assert max(counts) >= 3  # the cases reach chains of several matches


def test_hausdorff_and_euclidean_definitions(oracle):
    for a, b in _cases(40, 4, hi=12):
        assert oracle.pair("hausdorff", a, b) == hausdorff_def(a, b)
        assert oracle.pair("euclidean", a, b) == euclid_def(a, b)
