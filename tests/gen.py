"""Seeded synthetic layouts with the shapes of the benchmark configurations.

cfg0-style: lower-left uniform in a square die, width/height uniform ints in
[20, 2000] (about 30% of boxes overlap another at N=100k in a 1e6 die).
"""
import numpy as np


def random_layer(n, die=1_000_000, wmin=20, wmax=2000, seed=0, x0=0, y0=0):
    rng = np.random.default_rng(seed)
    w = rng.integers(wmin, wmax + 1, n)
    h = rng.integers(wmin, wmax + 1, n)
    x = rng.integers(0, max(1, die - w)) if n == 0 else rng.integers(0, np.maximum(1, die - w))
    y = rng.integers(0, np.maximum(1, die - h))
    b = np.stack([x + x0, y + y0, x + x0 + w, y + y0 + h], axis=1).astype(np.int32)
    return b


def cells_layout(ncell, median=8000, sigma=0.92, lo=100, hi=200_000, seed=2, scale=1.0):
    """Batched deck cells: lognormal box counts, each cell a cfg0-style layer
    in a die scaled to its box count (side 1e6*sqrt(n/1e5))."""
    rng = np.random.default_rng(seed)
    counts = np.clip(np.round(rng.lognormal(np.log(median * scale), sigma, ncell)), lo, hi).astype(np.int64)
    parts = []
    for k, n in enumerate(counts):
        die = int(1_000_000 * np.sqrt(n / 100_000.0))
        parts.append(random_layer(int(n), die=max(die, 4000), seed=seed * 100003 + k))
    off = np.zeros(ncell + 1, np.int64)
    off[1:] = np.cumsum(counts)
    return np.concatenate(parts), off
