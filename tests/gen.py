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


def stdcell_layers(n_per_layer, die=200_000, seed=1):
    """Standard-cell-style layers: rows 2720 dbu tall; poly vertical stripes
    150 wide on 340-pitch tracks (lengths 500..2500); met1 horizontal and met2
    vertical wires 140 wide (lengths round(lognormal(7, 1))); li1 random
    rects 170..800; 2% contacts 170x170."""
    rng = np.random.default_rng(seed)
    n = n_per_layer
    tracks = die // 340
    px = rng.integers(0, tracks, n) * 340
    py = rng.integers(0, die - 2600, n)
    pl = rng.integers(500, 2501, n)
    poly = np.stack([px, py, px + 150, py + pl], 1)
    L = np.clip(np.round(rng.lognormal(7, 1, n)), 140, die // 2).astype(np.int64)
    mx = rng.integers(0, die - L)
    my = rng.integers(0, die // 340, n) * 340
    met1 = np.stack([mx, my, mx + L, my + 140], 1)
    L2 = np.clip(np.round(rng.lognormal(7, 1, n)), 140, die // 2).astype(np.int64)
    nx = rng.integers(0, die // 340, n) * 340 + 100
    ny = rng.integers(0, die - L2)
    met2 = np.stack([nx, ny, nx + 140, ny + L2], 1)
    w = rng.integers(170, 801, n)
    h = rng.integers(170, 801, n)
    lx = rng.integers(0, die - w)
    ly = rng.integers(0, die - h)
    li1 = np.stack([lx, ly, lx + w, ly + h], 1)
    nc = max(1, n // 50)
    cx = rng.integers(0, die - 170, nc)
    cy = rng.integers(0, die - 170, nc)
    cont = np.stack([cx, cy, cx + 170, cy + 170], 1)
    return {k: v.astype(np.int32) for k, v in
            dict(poly=poly, met1=met1, met2=met2, li1=li1, contact=cont).items()}


def macro_arrays(nmacro=4, seed=3, pitch=400, size=200, side=64):
    """Full-chip macro blocks: side x side arrays of identical size x size
    boxes at the given pitch, at random non-overlapping-ish offsets."""
    rng = np.random.default_rng(seed)
    parts = []
    for m in range(nmacro):
        ox = int(rng.integers(0, 8)) * side * pitch + 1000 * m
        oy = int(rng.integers(0, 8)) * side * pitch
        ii, jj = np.meshgrid(np.arange(side), np.arange(side))
        x = ox + ii.ravel() * pitch
        y = oy + jj.ravel() * pitch
        parts.append(np.stack([x, y, x + size, y + size], 1))
    return np.concatenate(parts).astype(np.int32)
