"""Seeded synthetic TSP instances (integer coordinates stored as float32).

The reference was run on TSPLIB files (release/acouav*.sh); the workloads
here are synthetic stand-ins with the same shapes: uniform integer
coordinates, or Gaussian clusters rounded to integers.  The stream is
SplitMix64 (Steele, Lea & Flood 2014) seeded per instance, so an instance is
a pure function of (kind, n, seed).
"""
import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z):
    z = z.copy()
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


class SplitMix64:
    def __init__(self, seed):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def next_u64(self, count):
        with np.errstate(over="ignore"):
            idx = np.arange(1, count + 1, dtype=np.uint64)
            states = self.state + idx * _GOLDEN
            self.state = self.state + np.uint64(count) * _GOLDEN
        return _mix64(states)

    def uniform(self, count):
        """Doubles in [0, 1) with 53 random bits."""
        return (self.next_u64(count) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)

    def integers(self, count, high):
        return np.minimum((self.uniform(count) * high).astype(np.int64), high - 1)

    def normal(self, count):
        u1 = self.uniform(count)
        u2 = self.uniform(count)
        return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


def uniform_instance(n, box=10000, seed=1):
    """n cities with integer coordinates uniform in [0, box)^2."""
    g = SplitMix64(seed)
    xy = g.integers(2 * n, box).reshape(n, 2)
    return xy[:, 0].astype(np.float32), xy[:, 1].astype(np.float32)


def clustered_instance(n, box=10000, clusters=20, sigma=300.0, seed=1):
    """n cities drawn around `clusters` centres uniform in [0, box)^2 with
    N(0, sigma^2) offsets, rounded to integers; points outside the box are
    redrawn."""
    g = SplitMix64(seed)
    centres = g.uniform(2 * clusters).reshape(clusters, 2) * box
    pts = np.empty((0, 2), dtype=np.int64)
    while len(pts) < n:
        need = n - len(pts)
        cid = g.integers(need, clusters)
        off = g.normal(2 * need).reshape(need, 2) * sigma
        p = np.rint(centres[cid] + off).astype(np.int64)
        ok = (p >= 0).all(axis=1) & (p < box).all(axis=1)
        pts = np.concatenate([pts, p[ok]])
    pts = pts[:n]
    return pts[:, 0].astype(np.float32), pts[:, 1].astype(np.float32)


def euc2d_distances(x, y):
    """EUC_2D rounded distances with 0x7fffffff on the diagonal, computed like
    the reference (float differences, double root; src/Utils.cu:212-218)."""
    x = np.asarray(x, dtype=np.float32)
    y = np.asarray(y, dtype=np.float32)
    xd = (x[:, None] - x[None, :]).astype(np.float64)
    yd = (y[:, None] - y[None, :]).astype(np.float64)
    d = (np.sqrt(xd * xd + yd * yd) + 0.5).astype(np.int32)
    np.fill_diagonal(d, 0x7FFFFFFF)
    return d


def batch_sizes(count, lo=50, hi=2000, seed=7):
    """Instance sizes log-uniform in [lo, hi] (rounded)."""
    g = SplitMix64(seed)
    u = g.uniform(count)
    return np.rint(np.exp(np.log(lo) + u * (np.log(hi) - np.log(lo)))).astype(np.int64)
