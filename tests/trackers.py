"""Tracker (corner token) sets for the event-sort tests and golden fixtures.

The tracker layout is the reference's XYTracker (event_sorter.cu:15-19):
int32 X, int32 Y, int8 polygonNumber, padded to 12 bytes.
"""
import hashlib

import numpy as np

TRACKER_DTYPE = np.dtype([("X", np.int32), ("Y", np.int32), ("polygonNumber", np.int8), ("pad", np.int8, 3)])


def corner_trackers(b):
    """Four corner tokens per box with the signs of generate_trackers
    (polygon_fracture.f90:767-803): +1 at (x1,y1) and (x2,y2), -1 at (x1,y2)
    and (x2,y1)."""
    b = np.asarray(b, np.int32).reshape(-1, 4)
    t = np.zeros(4 * len(b), TRACKER_DTYPE)
    t["X"] = np.stack([b[:, 0], b[:, 0], b[:, 2], b[:, 2]], 1).ravel()
    t["Y"] = np.stack([b[:, 1], b[:, 3], b[:, 1], b[:, 3]], 1).ravel()
    t["polygonNumber"] = np.tile(np.array([1, -1, -1, 1], np.int8), len(b))
    return t


def seeded_trackers(n=200_000, seed=17, lo=-50000, hi=50000):
    rng = np.random.default_rng(seed)
    t = np.zeros(n, TRACKER_DTYPE)
    t["X"] = rng.integers(lo, hi, n)
    t["Y"] = rng.integers(lo, hi, n)
    t["polygonNumber"] = rng.choice(np.array([-1, 1], np.int8), n)
    return t


def as_rows(t):
    """(X, Y, polygonNumber) rows, int64."""
    return np.stack([t["X"].astype(np.int64), t["Y"].astype(np.int64), t["polygonNumber"].astype(np.int64)], 1)


def canonical_digest(t):
    """SHA-256 of (X, Y, polygonNumber) sorted by (X, Y, polygonNumber): equal
    for two sorts that agree on the keys and on the payload multiset per key."""
    o = np.lexsort((t["polygonNumber"], t["Y"], t["X"]))
    return hashlib.sha256(np.ascontiguousarray(as_rows(t[o]), "<i8").tobytes()).hexdigest()


def check_sorted_like(got, ref_rows):
    """got (a tracker array) has the reference's key order and, per key, the
    reference's multiset of payloads."""
    g = as_rows(got)
    r = np.asarray(ref_rows, np.int64).reshape(-1, 3)
    if len(g) != len(r) or not np.array_equal(g[:, :2], r[:, :2]):
        return False
    og = np.lexsort((g[:, 2], g[:, 1], g[:, 0]))
    orr = np.lexsort((r[:, 2], r[:, 1], r[:, 0]))
    return np.array_equal(g[og], r[orr])
