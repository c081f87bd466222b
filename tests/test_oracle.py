"""CPU tests: the oracle against the reference's known answers, its own
fixtures (tests/golden, generated from the reference by make_golden.py), an
independent brute-force restatement, and point-set identities."""
import json
import os

import numpy as np
import pytest

from bruteforce import canonical as brute
from gen import random_layer

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.json")


def test_known_answer_klee_175(oracle):
    # klee.cu:212-227: {0,0,10,10} and {5,5,15,15} -> union area 175
    assert oracle.union_area([[0, 0, 10, 10], [5, 5, 15, 15]]) == 175


def test_known_answer_and(oracle):
    # thrust_boolean.cu:494-549: (0,0,10,10) AND (5,5,20,20) -> (5,5,10,10)
    r = oracle.boolean([[0, 0, 10, 10]], [[5, 5, 20, 20]], oracle.AND)
    assert r.tolist() == [[5, 5, 10, 10]]


def test_known_answer_box_minus_hole(oracle):
    # test_rectboolean.f90:37-54: (0,0,10,10) minus (2,2,8,8) -> 4 fragments, area 64
    r = oracle.boolean([[0, 0, 10, 10]], [[2, 2, 8, 8]], oracle.NOT)
    assert len(r) == 4 and oracle.area_of(r) == 64
    # the fragments are left, right, bottom-middle, top-middle (rectboolean.f90:128-181)
    assert sorted(map(tuple, r.tolist())) == [(0, 0, 2, 10), (2, 0, 8, 2), (2, 8, 8, 10), (8, 0, 10, 10)]


def test_um_to_dbu_truncates(oracle):
    # controlparser.f90:146,568-576: int(1000*r) truncates toward zero
    assert oracle.um_to_dbu(0.001) == 1
    assert oracle.um_to_dbu(-0.001) == -1
    assert oracle.um_to_dbu(0.0045) == 4
    assert oracle.um_to_dbu(-0.0045) == -4


def _golden():
    with open(GOLDEN) as fh:
        return json.load(fh)["fixtures"]


@pytest.mark.parametrize("name", sorted(_golden().keys()))
def test_golden_fixture(oracle, name):
    rec = _golden()[name]
    b = np.array(rec["boxes"], np.int32).reshape(-1, 4)
    m = oracle.merge(b) if len(b) else np.zeros((0, 4), np.int32)
    assert m.tolist() == rec["merge"]
    # healed layer invariant (magparser.f90:433-443): sum of strip areas == union area
    assert oracle.area_of(m) == rec["union_area"] == oracle.union_area(b)
    assert oracle.components(b)[0] == rec["components"]
    if len(b) and "ref_morton_sorted_keys" in rec:
        keys = np.sort(oracle.morton_keys_np(b))
        assert keys.tolist() == rec["ref_morton_sorted_keys"] == rec["ref_morton_indirect_keys"]
        assert oracle.morton_keys(b).tolist() == oracle.morton_keys_np(b).tolist()
    if len(b):
        counts, area = oracle.op1(b, 1)
        assert counts["ring_and1"] == 0 and counts["ring_intersection"] == 0
        assert area == rec["union_area"]


def test_oracle_tracker_order_matches_reference(oracle):
    """The oracle's tracker key (PackKeys, event_sorter.cu:48-59) orders the
    fixtures' corner tokens as the reference's own cpp_std_sort_trackers did
    (keys, and the payload multiset per key), and the seeded set's digest."""
    from trackers import canonical_digest, check_sorted_like, corner_trackers, seeded_trackers
    with open(GOLDEN) as fh:
        g = json.load(fh)
    for name, rec in g["fixtures"].items():
        if "ref_sorted_trackers" not in rec:
            continue
        t = corner_trackers(np.array(rec["boxes"], np.int32).reshape(-1, 4))
        k = oracle.tracker_keys_np(t["X"], t["Y"])
        assert check_sorted_like(t[np.argsort(k, kind="stable")], rec["ref_sorted_trackers"]), name
    sg = g["seeded_trackers"]
    t = seeded_trackers(sg["n"], sg["seed"], *sg["x_range"])
    k = oracle.tracker_keys_np(t["X"], t["Y"])
    assert canonical_digest(t[np.argsort(k, kind="stable")]) == sg["sha256"]


def test_golden_provenance():
    """The golden file says which values come from the reference's code."""
    with open(GOLDEN) as fh:
        g = json.load(fh)
    assert "ref_sorted_trackers" in g["provenance"]["reference"]
    assert set(g["provenance"]["oracle"]) == {"merge", "union_area", "components"}


def test_square_fixture_areas(oracle):
    rec = _golden()["square_L68_D20.bin"]
    b = np.array(rec["boxes"], np.int32)
    assert oracle.area_of(b) == 3400 and rec["union_area"] == 3400


def test_complement_identity(oracle):
    # test_polygonfracture.f90:147-193: complement inside bbox+1000 has area bbox - layer
    b = random_layer(300, die=20000, seed=3)
    bb = [int(b[:, 0].min()) - 1000, int(b[:, 1].min()) - 1000, int(b[:, 2].max()) + 1000,
          int(b[:, 3].max()) + 1000]
    comp = oracle.boolean([bb], b, oracle.NOT)
    box_area = (bb[2] - bb[0]) * (bb[3] - bb[1])
    assert oracle.area_of(comp) == box_area - oracle.union_area(b)


@pytest.mark.parametrize("op", [0, 1, 2, 3, 4, 7])
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_oracle_matches_bruteforce(oracle, op, seed):
    A = random_layer(40, die=3000, wmin=5, wmax=600, seed=seed, x0=-1500)
    B = random_layer(40, die=3000, wmin=5, wmax=600, seed=seed + 50, y0=-800)
    for g in (16, 13, 10):
        r = oracle.boolean(A, B, op, g)
        assert r.tolist() == brute(A, B, op, g).tolist()


@pytest.mark.parametrize("g", [16, 14, 13])
def test_grow_and_dilation_match_bruteforce(oracle, g):
    """GROW (box_grow_directional, then heal) and SIZE +s (Minkowski dilation of
    the union = union of the dilated boxes) on the tile grids the slab-height
    tuner chooses from: the union of the moved boxes, rasterised independently."""
    A = random_layer(60, die=40000, wmin=5, wmax=3000, seed=g, x0=-20000, y0=-9000)
    for E, N, W, S in ((3, 1, 2, 5), (700, 0, 0, 1300)):
        G = A.astype(np.int64) + np.array([-W, -S, E, N])
        assert oracle.grow(A, E, N, W, S, g).tolist() == brute(G, G[:0], 4, g).tolist()
    for s_ in (1, 2500):
        D = A.astype(np.int64) + np.array([-s_, -s_, s_, s_])
        assert oracle.size(A, s_, g).tolist() == brute(D, D[:0], 4, g).tolist()


def test_point_set_identities(oracle):
    A = random_layer(2000, die=200000, seed=7)
    B = random_layer(2000, die=200000, seed=8)
    a, b = oracle.union_area(A), oracle.union_area(B)
    u = oracle.area_of(oracle.boolean(A, B, oracle.OR))
    i = oracle.area_of(oracle.boolean(A, B, oracle.AND))
    d = oracle.area_of(oracle.boolean(A, B, oracle.NOT))
    x = oracle.area_of(oracle.boolean(A, B, oracle.XOR))
    assert u + i == a + b and d + i == a and x == u - i
    # the decomposition does not depend on the input decomposition
    assert oracle.xor_empty(oracle.merge(A), A)
    assert oracle.merge(oracle.merge(A)).tolist() == oracle.merge(A).tolist()
    # the grid changes the cut lines, never the point set
    assert oracle.area_of(oracle.merge(A, 12)) == a
    assert oracle.xor_empty(oracle.merge(A, 12), oracle.merge(A, 16))


def test_size_semantics(oracle):
    assert oracle.size([[0, 0, 10, 10]], -1).tolist() == [[1, 1, 9, 9]]
    assert len(oracle.size([[0, 0, 2, 2]], -1)) == 0
    assert oracle.size([[0, 0, 10, 10], [10, 0, 20, 10]], -2).tolist() == [[2, 2, 18, 8]]
    A = random_layer(1500, die=100000, seed=11)
    for s in (1, 3, 40):
        er = oracle.size(A, -s)
        # erosion then dilation stays inside the original (opening)
        back = oracle.size(er, s) if len(er) else er
        assert len(oracle.boolean(back, A, oracle.NOT)) == 0
        # dilation contains the original
        assert len(oracle.boolean(A, oracle.size(A, s), oracle.NOT)) == 0


def test_components_semantics(oracle):
    # closed overlap (pnummerge.f90:341-342): edge and corner touches connect
    n, lab = oracle.components([[0, 0, 1, 1], [1, 1, 2, 2], [5, 5, 6, 6], [1, 0, 3, 1]])
    assert n == 2 and lab.tolist() == [1, 1, 0, 1]
    n, lab = oracle.components([[0, 0, 1, 1]])
    assert n == 1 and lab.tolist() == [0]
    n, lab = oracle.components([[10, 10, 20, 20], [0, 0, 5, 5], [4, 4, 11, 11]])
    assert n == 1 and lab.tolist() == [1, 1, 1]


def test_overlap_semantics(oracle):
    # CalculateSingleLayerAND (design_impl.f90:385-498): positive-area pairwise
    # intersections, as a point set the area covered at least twice
    A = [[0, 0, 10, 10], [5, 5, 15, 15], [10, 0, 20, 5], [30, 30, 40, 40], [30, 30, 40, 40]]
    assert oracle.overlap(A).tolist() == [[5, 5, 10, 10], [30, 30, 40, 40]]
    assert len(oracle.overlap([[0, 0, 1, 1], [1, 0, 2, 1]])) == 0  # edge touch only
    B = random_layer(3000, die=300000, seed=21)
    # a healed layer overlaps nowhere; overlap lies inside the union
    assert len(oracle.overlap(oracle.merge(B))) == 0
    assert len(oracle.boolean(oracle.overlap(B), oracle.merge(B), oracle.NOT)) == 0


def _pairs_brute(A):
    A = np.asarray(A, np.int64)
    n = len(A)
    strict = 0
    touched = np.zeros(n, bool)
    for i in range(n):
        for k in range(i + 1, n):
            ox = max(A[i, 0], A[k, 0]), min(A[i, 2], A[k, 2])
            oy = max(A[i, 1], A[k, 1]), min(A[i, 3], A[k, 3])
            if ox[0] <= ox[1] and oy[0] <= oy[1]:
                touched[i] = touched[k] = True
                strict += ox[0] < ox[1] and oy[0] < oy[1]
    return strict, int((~touched).sum()), (~touched).astype(np.uint8)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_interactions_match_bruteforce(oracle, seed):
    # ComputeInteractionsCPU (pnummerge.f90:483-562, strict <) and
    # FindSingletonsCPU (:388-482, closed <=)
    A = random_layer(300, die=20000, wmin=5, wmax=900, seed=seed)
    A = np.concatenate([A, A[:5], [[0, 0, 10, 10], [10, 0, 20, 10], [20, 10, 30, 20]]]).astype(np.int32)
    p, s, m = oracle.interactions(A)
    ep, es, em = _pairs_brute(A)
    assert (p, s) == (ep, es) and m.tolist() == em.tolist()
    # a healed layer certifies: no strict pairs
    assert oracle.interactions(oracle.merge(A))[0] == 0


def test_component_areas(oracle):
    A = [[0, 0, 10, 10], [5, 5, 15, 15], [20, 0, 30, 10], [30, 0, 40, 10], [100, 100, 110, 110]]
    assert oracle.component_areas(A).tolist() == [100, 175, 200]
    B = random_layer(5000, die=400000, seed=9)
    ar = oracle.component_areas(B)
    n, lab = oracle.components(B)
    assert len(ar) == lab.max() + 1 and ar.sum() == oracle.union_area(B)


def test_refpath_subtract_known_answer(oracle):
    # SubtractBox (boolean_ops_rtree.f90:139-186) on the box-minus-hole case of
    # test_rectboolean.f90:37-54: left, right, bottom-middle, top-middle, area 64
    r = oracle.refpath_subtract([0, 0, 10, 10], [2, 2, 8, 8])
    assert r.tolist() == [[0, 0, 2, 10], [8, 0, 10, 10], [2, 0, 8, 2], [2, 8, 8, 10]]
    assert oracle.area_of(r) == 64
    assert oracle.refpath_subtract([0, 0, 10, 10], [10, 0, 20, 10]).tolist() == [[0, 0, 10, 10]]  # edge touch
    assert len(oracle.refpath_subtract([2, 2, 8, 8], [0, 0, 10, 10])) == 0


@pytest.mark.parametrize("n,die,seed", [(600, 60000, 61), (5000, 250000, 62)])
def test_refpath_op1_point_sets(oracle, n, die, seed):
    """The reference's CPU path for OP1 (FRAME tiles, R-tree AND clips,
    fracture NOT) gives the oracle's point sets for every layer (the
    decompositions differ), and both ASSERT_ZERO layers are empty."""
    A = random_layer(n, die=die, seed=seed)
    exp = [oracle.grow(A, 1, 1, 1, 1), oracle.size(A, -1)]
    exp.append(oracle.boolean(exp[0], A, oracle.NOT))
    exp.append(oracle.boolean(A, exp[1], oracle.NOT))
    for w in range(4):
        got = oracle.refpath_op1_layer(A, w)
        assert np.array_equal(oracle.merge(got), exp[w]), w
        assert oracle.area_of(got) == oracle.area_of(exp[w]), w  # the pieces are disjoint
    assert len(oracle.refpath_op1_layer(A, 4)) == 0 and len(oracle.refpath_op1_layer(A, 5)) == 0
    off = np.array([0, n], np.int64)
    counts, area = oracle.refpath_op1_cells(A, off)
    assert counts[0, 4] == 0 and counts[0, 5] == 0 and area[0] == oracle.union_area(A)


def test_strip_digest_formula(oracle):
    """The per-cell strip digest (gb_layer_digest on the device, orc_strip_digest
    in the oracle) is the sum mod 2^64 of fmix64((x1<<32|y1) ^ fmix64((x2<<32|y2)
    + 0x9e3779b97f4a7c15)) over the strips, coordinates as uint32; it does not
    depend on the strip order."""
    M = (1 << 64) - 1

    def fmix(k):
        k ^= k >> 33
        k = (k * 0xff51afd7ed558ccd) & M
        k ^= k >> 33
        k = (k * 0xc4ceb9fe1a85ec53) & M
        return k ^ (k >> 33)

    def h(x1, y1, x2, y2):
        u = ((x1 & 0xffffffff) << 32) | (y1 & 0xffffffff)
        v = ((x2 & 0xffffffff) << 32) | (y2 & 0xffffffff)
        return fmix(u ^ fmix((v + 0x9e3779b97f4a7c15) & M))

    b = random_layer(500, die=40000, seed=71, x0=-20000)
    assert oracle.strip_digest(b) == sum(h(*map(int, r)) for r in b) & M
    assert oracle.strip_digest(b[::-1]) == oracle.strip_digest(b)
    assert oracle.strip_digest(b[:0]) == 0
    assert oracle.lib().orc_strip_hash(-1, 2, 3, -4) == h(-1, 2, 3, -4)
