"""Layers for the SNAP codec tests (CPU and GPU): the golden fixtures and
seeded layers covering what the codec distinguishes -- squares, repeated and
new widths / heights, anchor deltas of both signs and of int32 extremes,
widths that wrap int32, chunk boundaries, dictionaries larger than a
shared-memory table, and more than 32767 distinct widths in one chunk (an
int16 index the reference cannot decode)."""
import base64
import hashlib
import json
import os

import numpy as np

import gen

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "snap_golden.json")


def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


def golden_layers():
    """[(name, boxes, [(num_boxes, raw_byte_size, raw_sha256, library_snappy_bytes)])]"""
    g = golden()
    out = []
    for name, rec in g["fixtures"].items():
        b = np.array(rec["boxes"], np.int32).reshape(-1, 4)
        out.append((name, b, _chunks(rec["chunks"])))
    for name, rec in g["synthetic"].items():
        fn = getattr(gen, rec["generator"])
        B = fn(**rec["args"])
        if isinstance(B, dict):
            B = np.concatenate([B[k] for k in ("poly", "met1", "met2", "li1", "contact")])
        out.append((name, B, _chunks(rec["chunks"]), rec["sha256"]))
    return out


def _chunks(recs):
    return [(c["num_boxes"], c["raw_byte_size"], c["raw_sha256"], base64.b64decode(c["snappy_library"]))
            for c in recs]


def sha(A):
    return hashlib.sha256(np.ascontiguousarray(A, "<i4").tobytes()).hexdigest()


def cases(big=False):
    """Named seeded layers (boxes valid: x1 < x2, y1 < y2)."""
    rng = np.random.default_rng(7)
    c = {}
    c["one"] = np.array([[3, 4, 5, 9]], np.int32)
    c["one_square"] = np.array([[-3, -4, 5, 4]], np.int32)
    c["identical"] = np.repeat(np.array([[10, 20, 30, 40]], np.int32), 1000, axis=0)
    c["random_5000"] = gen.random_layer(5000, seed=1)
    c["squares"] = np.stack([np.arange(3000) * 7, np.arange(3000) % 13, np.arange(3000) * 7 + 5,
                             np.arange(3000) % 13 + 5], 1).astype(np.int32)
    ext = np.array([[-2147483648, -2147483648, -2147483647, 2147483647],
                    [2147483646, -5, 2147483647, 5],
                    [-2000000000, 7, 2000000000, 9],        # width 4e9 wraps int32
                    [0, -2000000000, 3, 2000000000],        # height wraps
                    [-2147483648, 0, 2147483647, 1],
                    [5, 5, 6, 6]], np.int32)
    c["extremes"] = np.concatenate([ext, ext[::-1], ext])
    sc = gen.stdcell_layers(2000, seed=3)
    c["stdcell"] = np.concatenate([sc[k] for k in ("poly", "met1", "met2", "li1", "contact")])
    c["chunk_exact"] = gen.random_layer(65536, seed=4)
    c["chunk_plus_one"] = gen.random_layer(65537, seed=5)
    # about 5000 distinct widths in one chunk (a shared-memory table), and
    # about 17000 (more than it holds: the global-memory table)
    for name, wmax, nbx in (("many_widths", 5001, 20000), ("more_widths", 30001, 30000)):
        w = rng.integers(1, wmax, nbx)
        h = rng.integers(1, 300, nbx)
        x = rng.integers(-1000000, 1000000, nbx)
        y = rng.integers(-1000000, 1000000, nbx)
        c[name] = np.stack([x, y, x + w, y + h], 1).astype(np.int32)
    if big:
        c["macros"] = gen.macro_arrays(nmacro=40, seed=9)
        c["random_300k"] = gen.random_layer(300000, seed=6)
    return c


def wrap_case():
    """40000 distinct widths in one chunk: indices above 32767 wrap in the
    int16 field, which the reference's decoder rejects as a desync."""
    n = 50000
    i = np.arange(n)
    w = np.where(i < 40000, i + 1, 33001 + (i - 40000) % 7000)  # then reuse indices 33001..40000
    x = i * 3
    return np.stack([x, np.zeros(n), x + w, np.full(n, 10)], 1).astype(np.int32)
