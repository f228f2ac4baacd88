"""Seeded synthetic trajectory generators.

There is no public dataset behind any workload of this engine: every input is
a seeded random walk with the shapes and distributions of the workloads it
stands for.  Trajectory sets are CSR: ``pts`` float32 [total, 2] (x, y per
point, the reference's ``struct Point``) and ``off`` int64 [count + 1].
"""
from __future__ import annotations

import numpy as np


def csr_from_lengths(lengths):
    lengths = np.asarray(lengths, np.int64)
    off = np.zeros(len(lengths) + 1, np.int64)
    np.cumsum(lengths, out=off[1:])
    return off


def random_walks(count: int, lengths, seed: int, *, start_range: float = 100.0,
                 step: str = "normal", nu: float = 3.0):
    """``count`` 2-D random walks: start uniform in [0, start_range)^2, steps
    N(0,1) per coordinate (``step="normal"``) or Student-t with ``nu`` degrees
    of freedom (``step="student_t"``).  ``lengths`` is an int or an array."""
    rng = np.random.default_rng(seed)
    if np.isscalar(lengths):
        lengths = np.full(count, int(lengths), np.int64)
    lengths = np.asarray(lengths, np.int64)
    off = csr_from_lengths(lengths)
    total = int(off[-1])
    if step == "normal":
        steps = rng.standard_normal((total, 2))
    else:
        steps = rng.standard_t(nu, (total, 2))
    starts = rng.uniform(0.0, start_range, (count, 2))
    steps[off[:-1]] = starts
    # cumulative sum restarted at each trajectory start
    cs = np.cumsum(steps, axis=0)
    base = np.repeat(cs[off[:-1]] - starts, lengths, axis=0)
    pts = (cs - base).astype(np.float32)
    return pts, off


def uniform_lengths(count, lo, hi, seed):
    return np.random.default_rng(seed).integers(lo, hi + 1, count)


def lognormal_lengths(count, mu, sigma, lo, hi, seed):
    x = np.random.default_rng(seed).lognormal(mu, sigma, count)
    return np.clip(np.rint(x), lo, hi).astype(np.int64)


# ---------------------------------------------------------------- reference-style data
def ref_base_trajectories(num_t: int, n: int, seed: int, r: float = 1000.0):
    """Random walks with uniform steps in [-1, 1] clamped to [0, r], the
    shape CudaRuntime1/main.cu:12-33 generates (seeded numpy instead of
    rand()).  Returns a fixed-length AoS array [num_t * n, 2]."""
    rng = np.random.default_rng(seed)
    t = np.empty((num_t, n, 2), np.float32)
    t[:, 0] = rng.uniform(0, r, (num_t, 2))
    steps = rng.uniform(-1.0, 1.0, (num_t, n, 2)).astype(np.float32)
    for i in range(1, n):
        t[:, i] = np.clip(t[:, i - 1] + steps[:, i], 0.0, r)
    return t.reshape(num_t * n, 2)


def ref_similar_trajectories(t1, num_t: int, n: int, m: int, noise: float, seed: int,
                             r: float = 1000.0):
    """Noisy resampling of each t1 trajectory to length m, the shape
    CudaRuntime1/main.cu:34-64 generates: trajectory k of t2 is a noisy copy
    of trajectory k of t1."""
    rng = np.random.default_rng(seed)
    t1 = np.asarray(t1, np.float32).reshape(num_t, n, 2)
    if m > 1:
        src = np.rint(np.arange(m, dtype=np.float32) * (n - 1) / (m - 1)).astype(np.int64)
    else:
        src = np.zeros(1, np.int64)
    src = np.clip(src, 0, n - 1)
    base = t1[:, src]
    nz = (rng.uniform(0, 1, (num_t, m, 2)) * noise * 2.0 - noise).astype(np.float32)
    return np.clip(base + nz, 0.0, r).astype(np.float32).reshape(num_t * m, 2)
