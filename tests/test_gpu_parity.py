"""GPU parity: every operator of the CUDA path against the oracle, bit-exact
after canonical ordering, on seeded inputs, the reference fixtures and the
edge cases of the domain.  All calls go through the C-ABI (libgbool.so)."""
import json
import os

import numpy as np
import pytest

from gen import cells_layout, random_layer

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.json")
OPS = [0, 1, 2, 3]


def canon(b):
    b = np.asarray(b, np.int32).reshape(-1, 4)
    if len(b) == 0:
        return b
    return b[np.lexsort((b[:, 3], b[:, 2], b[:, 1], b[:, 0]))]


def gpu_bool(ctx, A, B, op):
    m = ctx.mark()
    try:
        LA, LB = ctx.layer(A), ctx.layer(B)
        out = ctx.op(op, LA, LB) if op != 4 else ctx.op(4, LA)
        res = out.to_numpy()
        LA.free()
        LB.free()
        return canon(res)
    finally:
        ctx.release(m)


def check(ctx, oracle, A, B, op):
    got = gpu_bool(ctx, A, B, op)
    exp = oracle.boolean(A, B, op) if op != 4 else oracle.merge(A)
    assert got.shape == exp.shape, (got.shape, exp.shape)
    assert np.array_equal(got, exp)


CASES = {
    "small": lambda: (random_layer(200, die=20000, seed=1), random_layer(200, die=20000, seed=2)),
    "cross_tiles": lambda: (random_layer(20000, die=400000, seed=3, x0=-200000, y0=-70000),
                            random_layer(20000, die=400000, seed=4, x0=-200000, y0=-70000)),
    "dense": lambda: (random_layer(4000, die=30000, seed=5), random_layer(4000, die=30000, seed=6)),
    "cfg0_like": lambda: (random_layer(100000, seed=7), random_layer(100000, seed=8)),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("op", OPS + [4])
def test_bool_parity(ctx, oracle, case, op):
    A, B = CASES[case]()
    check(ctx, oracle, A, B, op)


def test_edge_cases(ctx, oracle):
    one = np.array([[0, 0, 10, 10]], np.int32)
    empty = np.zeros((0, 4), np.int32)
    big = np.array([[-100000, -100000, 200000, 200000]], np.int32)  # spans 5x5 tiles
    for A, B in [(one, empty), (empty, one), (one, one), (big, one), (one, big),
                 (np.repeat(one, 7, axis=0), one),  # exact duplicates (SED_L122_D16 has some)
                 (np.array([[0, 0, 5, 5], [5, 0, 10, 5], [0, 5, 5, 10]], np.int32), one),  # edge touches
                 (np.array([[65535, 65535, 65537, 65537]], np.int32), one),  # straddles a tile corner
                 (np.array([[-2000000000, -2000000000, -1999990000, -1999990000]], np.int32),
                  np.array([[-1999000000, -1999995000, -1998000000, -1999993000]], np.int32)),
                 (np.array([[-2000000, -2000000, -1990000, -1990000]], np.int32), big)]:
        for op in OPS + [4]:
            check(ctx, oracle, A, B, op)
    # A XOR A is empty, A NOT A is empty
    A = random_layer(5000, die=150000, seed=9)
    assert len(gpu_bool(ctx, A, A, 0)) == 0
    assert len(gpu_bool(ctx, A, A, 3)) == 0


def test_tile_window_limit_is_an_error(ctx):
    """A cell whose tile window exceeds 2^28 tiles (boxes ~4e9 dbu apart at
    the default 65536-dbu grid) is refused with GB_ERR_CAPACITY, not run."""
    from vlsi_layout_gb300 import engine
    A = np.array([[-2147480000, -2147480000, -2147470000, -2147470000],
                  [2147400000, 2147400000, 2147410000, 2147410000]], np.int32)
    m = ctx.mark()
    try:
        with pytest.raises(engine.GBError) as ei:
            ctx.op(4, ctx.layer(A)).to_numpy()
        assert ei.value.code == engine.GB_ERR_CAPACITY
    finally:
        ctx.release(m)
    ctx.sync()  # the error was reported once and cleared


def test_golden_fixtures(ctx, oracle):
    with open(GOLDEN) as fh:
        fx = json.load(fh)["fixtures"]
    for name, rec in fx.items():
        b = np.array(rec["boxes"], np.int32).reshape(-1, 4)
        got = gpu_bool(ctx, b, np.zeros((0, 4), np.int32), 4)
        assert got.tolist() == rec["merge"], name


@pytest.mark.parametrize("s", [1, 3, 250])
def test_grow_size_parity(ctx, oracle, s):
    A = random_layer(20000, die=300000, seed=10 + s, x0=-65536)
    m = ctx.mark()
    try:
        L = ctx.layer(A)
        g = canon(ctx.grow(L, s, 2 * s, 3 * s, s).to_numpy())
        assert np.array_equal(g, oracle.grow(A, s, 2 * s, 3 * s, s))
        for sv in (s, -s):
            r = canon(ctx.size(L, sv).to_numpy())
            assert np.array_equal(r, oracle.size(A, sv)), sv
    finally:
        ctx.release(m)


def test_klee_area(ctx, oracle):
    for A in (np.array([[0, 0, 10, 10], [5, 5, 15, 15]], np.int32),  # klee.cu: 175
              random_layer(50000, die=500000, seed=12),
              random_layer(3000, die=40000, seed=13)):
        m = ctx.mark()
        L = ctx.layer(A)
        assert int(ctx.area(L)[0]) == oracle.union_area(A)
        ctx.release(m)


def test_components(ctx, oracle):
    for A in (random_layer(3000, die=60000, seed=14), random_layer(100000, seed=15),
              np.array([[0, 0, 1, 1], [1, 1, 2, 2], [5, 5, 6, 6], [1, 0, 3, 1]], np.int32),
              np.array([[0, 0, 1, 1]], np.int32)):
        n, lab = ctx.components(A)
        en, elab = oracle.components(A)
        assert n == en and np.array_equal(lab, elab)


def test_sorts(ctx, oracle):
    from vlsi_layout_gb300 import engine
    A = random_layer(300000, die=2_000_000, seed=16, x0=-1_000_000)
    # repeated boxes (equal Morton keys) at spread input positions, for the stability check
    rng = np.random.default_rng(16)
    A = np.concatenate([A, A[rng.integers(0, len(A), 20000)]])
    A = A[rng.permutation(len(A))]
    b, keys, perm = ctx.morton_sort(A)
    ek = oracle.morton_keys_np(A)
    assert np.array_equal(keys, np.sort(ek))
    assert np.array_equal(b, A[perm]) and np.array_equal(ek[perm], keys)
    assert np.array_equal(np.sort(perm), np.arange(len(A)))
    # stability of the LSD passes: within a run of equal keys the input order is kept
    eq = keys[1:] == keys[:-1]
    assert eq.sum() >= 20000 and np.all(perm[1:][eq] > perm[:-1][eq])
    d = engine.sort_boxes_direct(A)
    assert np.array_equal(oracle.morton_keys_np(d), np.sort(ek))
    idx = engine.sort_boxes_indirect(A)
    assert idx.min() == 1 and np.array_equal(oracle.morton_keys_np(A[idx - 1]), np.sort(ek))
    c = ctx.canonical_sort(A[::-1])
    assert np.array_equal(c, canon(A))


def test_event_sort_matches_reference():
    """device_event_sort against the reference's own cpp_std_sort_trackers
    (event_sorter.cu:86-115, compiled from the reference sources when the
    golden file was made): the same key order, the same payload multiset per
    key; and, the device sort being stable, exactly numpy's stable order."""
    from trackers import canonical_digest, check_sorted_like, corner_trackers, seeded_trackers
    from vlsi_layout_gb300 import engine
    with open(GOLDEN) as fh:
        g = json.load(fh)
    n = 0
    for name, rec in g["fixtures"].items():
        if "ref_sorted_trackers" not in rec:
            continue
        t = corner_trackers(np.array(rec["boxes"], np.int32).reshape(-1, 4))
        s = engine.event_sort(t)
        assert check_sorted_like(s, rec["ref_sorted_trackers"]), name
        o = np.lexsort((t["Y"], t["X"]))  # stable: payloads keep their input order per key
        assert np.array_equal(s["polygonNumber"], t["polygonNumber"][o]), name
        n += 1
    assert n >= 15  # the non-empty fixtures
    sg = g["seeded_trackers"]
    t = seeded_trackers(sg["n"], sg["seed"], *sg["x_range"])
    s = engine.event_sort(t)
    assert canonical_digest(s) == sg["sha256"]
    o = np.lexsort((t["Y"], t["X"]))
    for f in ("X", "Y", "polygonNumber"):
        assert np.array_equal(s[f], t[f][o]), f


def test_golden_morton_order(ctx):
    """The device Morton sort reproduces the key order of the reference's own
    thrust_sort_boxes_direct / _indirect on its KLBin fixtures (negative
    coordinates and duplicates included)."""
    from vlsi_layout_gb300 import engine
    with open(GOLDEN) as fh:
        fx = json.load(fh)["fixtures"]
    for name, rec in fx.items():
        b = np.array(rec["boxes"], np.int32).reshape(-1, 4)
        if len(b) == 0 or "ref_morton_sorted_keys" not in rec:
            continue
        _, keys, _ = ctx.morton_sort(b)
        assert keys.astype(np.uint64).tolist() == rec["ref_morton_sorted_keys"], name
        idx = engine.sort_boxes_indirect(b)
        _, k2, _ = ctx.morton_sort(b[idx - 1])
        assert k2.tolist() == rec["ref_morton_indirect_keys"], name


def test_dropin_ffi(oracle):
    from vlsi_layout_gb300 import engine
    A = random_layer(3000, die=100000, seed=18)
    B = random_layer(3000, die=100000, seed=19)
    for op in OPS:
        assert np.array_equal(canon(engine.boost_polygon_operation(A, B, op)), oracle.boolean(A, B, op))
    assert np.array_equal(canon(engine.boost_polygon_operation(A, B, 4)), oracle.merge(A))
    assert np.array_equal(canon(engine.boost_polygon_operation(A, B, 5, -2)), oracle.size(A, -2))
    assert np.array_equal(canon(engine.boost_polygon_merge(A)), oracle.merge(A))
    assert len(engine.boost_polygon_operation(np.zeros((0, 4)), np.zeros((0, 4)), 1)) == 0


def test_multicell_layer(ctx, oracle):
    boxes, off = cells_layout(24, median=1500, seed=20)
    boxes2, _ = cells_layout(24, median=1500, seed=20)
    boxes2 = boxes2.copy()
    boxes2[:, [0, 2]] += 37
    m = ctx.mark()
    try:
        LA = ctx.layer(boxes, off)
        LB = ctx.layer(boxes2, off)
        for op in (2, 3, 0):
            res, coff = ctx.op(op, LA, LB).to_numpy(with_cells=True)
            for k in range(len(off) - 1):
                exp = oracle.boolean(boxes[off[k]:off[k + 1]], boxes2[off[k]:off[k + 1]], op)
                assert np.array_equal(canon(res[coff[k]:coff[k + 1]]), exp), (op, k)
    finally:
        ctx.release(m)


def test_op1_chain(ctx, oracle):
    """The OP1 chain op by op on a 100k-box cfg0-style layer: every one of the
    six result layers equals the oracle's strips (the oracle runs each
    operator on the previous operators' strips, as the deck does)."""
    A = random_layer(100000, seed=21)
    e_p1 = oracle.grow(A, 1, 1, 1, 1)
    e_p2 = oracle.size(A, -1)
    e_outer = oracle.boolean(e_p1, A, 3)
    e_inner = oracle.boolean(A, e_p2, 3)
    e_and1 = oracle.boolean(e_outer, A, 2)
    e_inter = oracle.boolean(e_outer, e_inner, 2)
    counts, area = oracle.op1(A, 1)
    m = ctx.mark()
    try:
        P = ctx.layer(A)
        p1 = ctx.grow(P, 1, 1, 1, 1)
        p2 = ctx.size(P, -1)
        outer = ctx.op(3, p1, P)
        inner = ctx.op(3, P, p2)
        and1 = ctx.op(2, outer, P)
        inter = ctx.op(2, outer, inner)
        for name, L, e in [("poly_1", p1, e_p1), ("poly_2", p2, e_p2), ("outer_ring", outer, e_outer),
                           ("inner_ring", inner, e_inner), ("ring_and1", and1, e_and1),
                           ("ring_intersection", inter, e_inter)]:
            assert np.array_equal(canon(L.to_numpy()), e), name
            assert L.count()[0] == counts[name] == len(e), name
            assert int(L.digest()[0]) == oracle.strip_digest(e), name
        assert len(e_and1) == 0 and len(e_inter) == 0
        assert int(ctx.area(P)[0]) == area
    finally:
        ctx.release(m)


def test_op1_cells_digest(ctx, oracle):
    """gb_op1 on a multi-cell layer: per cell, the digest of each result layer
    equals the oracle's digest of its strips for that cell (and the strips of a
    few cells are compared outright)."""
    boxes, off = cells_layout(64, median=4000, seed=22)
    ec, ea, ed = oracle.op1_cells_digest(boxes, off)
    m = ctx.mark()
    try:
        P = ctx.layer(boxes, off)
        outs = ctx.op1(P, 1)
        for j, L in enumerate(outs):
            assert np.array_equal(L.digest(), ed[:, j]), j
            assert np.array_equal(L.count()[1], ec[:, j]), j
        res, coff = outs[2].to_numpy(with_cells=True)  # outer ring, strip for strip on three cells
        for k in (0, 17, 63):
            A = boxes[off[k]:off[k + 1]]
            e = oracle.boolean(oracle.grow(A, 1, 1, 1, 1), A, 3)
            assert np.array_equal(canon(res[coff[k]:coff[k + 1]]), e), k
        merged = ctx.op(4, P)
        assert np.array_equal(merged.digest(), ed[:, 6])
    finally:
        ctx.release(m)


@pytest.mark.parametrize("amount", [1, 3, 0, -2])
def test_op1_area_cells(ctx, oracle, amount):
    """gb_op1_area: the chain's counts and the union area per cell (from the
    erosion's complement when amount > 0), with empty cells among them."""
    torch = pytest.importorskip("torch")
    from gen import cells_layout
    boxes, off = cells_layout(40, median=2000, seed=31 + amount)
    # make two cells empty
    keep = np.ones(len(boxes), bool)
    for k in (3, 17):
        keep[off[k]:off[k + 1]] = False
    sizes = np.diff(off) * np.array([0 if k in (3, 17) else 1 for k in range(len(off) - 1)])
    boxes = boxes[keep]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    m = ctx.mark()
    try:
        P = ctx.layer(boxes, off)
        area_t = torch.full((len(off) - 1,), -7, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        outs = ctx.op1_area(P, amount, area_t.data_ptr())
        ctx.sync()
        area = area_t.cpu().numpy()
        counts = np.stack([L.count()[1] for L in outs], axis=1)
    finally:
        ctx.release(m)
    if amount == 1:
        ec, ea = oracle.op1_cells(boxes, off)
        assert np.array_equal(counts, ec)
    else:
        ea = np.array([oracle.union_area(boxes[off[k]:off[k + 1]]) for k in range(len(off) - 1)])
    assert np.array_equal(area, ea)
    assert area[3] == 0 and area[17] == 0


def test_op1_host_two_groups(ctx, oracle):
    """gb_op1_host on a layout large enough to be split into two groups of cells
    (the second group's upload overlaps the first group's deck): per cell the
    strip digests of all six result layers, the counts and the union area equal
    the oracle's."""
    boxes, off = cells_layout(400, median=8000, seed=41)
    assert off[-1] >= (1 << 22)
    b = np.ascontiguousarray(boxes, np.int32)
    counts, area, fails, dig = ctx.op1_host(b.ctypes.data, len(b), off, 1, digests=True)
    ec, ea, ed = oracle.op1_cells_digest(b, off)
    assert np.array_equal(counts, ec) and np.array_equal(area, ea) and fails == 0
    assert np.array_equal(dig, ed[:, :6])
