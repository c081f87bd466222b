"""Single-layer AND (the area covered by at least two boxes of a layer,
CalculateSingleLayerAND, design_impl.f90:385-498), the overlap statistics of
the load-time PNUM loop (ComputeInteractionsCPU / FindSingletonsCPU,
pnummerge.f90:388-562, and CertifyHealing, design_impl.f90:35-56) and the
per-component union area (calculate_union_area_by_polygon,
design.f90:854-935) on the GPU, against the oracle."""
import os

import numpy as np
import pytest

from gen import cells_layout, macro_arrays, random_layer, stdcell_layers

pytestmark = pytest.mark.gpu


def canon(b):
    b = np.asarray(b, np.int32).reshape(-1, 4)
    return b[np.lexsort((b[:, 3], b[:, 2], b[:, 1], b[:, 0]))] if len(b) else b


def overlap_gpu(ctx, boxes, off=None):
    from vlsi_layout_gb300 import engine
    m = ctx.mark()
    try:
        L = ctx.layer(boxes, off) if off is not None else ctx.layer(boxes)
        return canon(ctx.op(engine.OVERLAP, L).to_numpy())
    finally:
        ctx.release(m)


def test_overlap_known_answers(ctx, oracle):
    A = np.array([[0, 0, 10, 10], [5, 5, 15, 15], [10, 0, 20, 5], [30, 30, 40, 40], [30, 30, 40, 40]], np.int32)
    assert overlap_gpu(ctx, A).tolist() == [[5, 5, 10, 10], [30, 30, 40, 40]]
    assert len(overlap_gpu(ctx, np.array([[0, 0, 1, 1], [1, 0, 2, 1]], np.int32))) == 0
    assert len(overlap_gpu(ctx, np.array([[0, 0, 100, 100]], np.int32))) == 0
    # three-deep stack: covered twice or more, across a tile boundary
    S = np.array([[65000, 0, 66000, 10], [65500, 0, 70000, 10], [65900, 5, 65950, 20]], np.int32)
    assert overlap_gpu(ctx, S).tolist() == [[65500, 0, 65536, 10], [65536, 0, 66000, 10]]
    assert oracle.overlap(S).tolist() == [[65500, 0, 65536, 10], [65536, 0, 66000, 10]]


@pytest.mark.parametrize("n,die,seed", [(20000, 1_000_000, 1), (60000, 600_000, 2), (5000, 40_000, 3)])
def test_overlap_random(ctx, oracle, n, die, seed):
    A = random_layer(n, die=die, seed=seed)
    assert np.array_equal(overlap_gpu(ctx, A), oracle.overlap(A))


def test_overlap_dense_shapes(ctx, oracle):
    L = stdcell_layers(30000, seed=4)
    for name in ("poly", "met1", "li1"):
        assert np.array_equal(overlap_gpu(ctx, L[name]), oracle.overlap(L[name])), name
    M = macro_arrays(nmacro=3, seed=5)
    D = np.concatenate([M, M[::7]])  # duplicated boxes overlap themselves exactly
    assert np.array_equal(overlap_gpu(ctx, D), oracle.overlap(D))


def test_overlap_cells(ctx, oracle):
    boxes, off = cells_layout(24, median=3000, seed=6)
    got = []
    from vlsi_layout_gb300 import engine
    m = ctx.mark()
    try:
        R = ctx.op(engine.OVERLAP, ctx.layer(boxes, off))
        res, roff = R.to_numpy(with_cells=True)
    finally:
        ctx.release(m)
    for k in range(len(off) - 1):
        exp = oracle.overlap(boxes[off[k]:off[k + 1]])
        assert np.array_equal(canon(res[roff[k]:roff[k + 1]]), exp), k


def test_overlap_of_healed_layer_is_empty(ctx, oracle):
    A = random_layer(30000, die=500_000, seed=8)
    healed = oracle.merge(A)
    assert len(overlap_gpu(ctx, healed)) == 0


@pytest.mark.parametrize("seed", [0, 1])
def test_interactions_random(ctx, oracle, seed):
    A = random_layer(50000, die=1_500_000, seed=seed)
    A = np.concatenate([A, A[:100], [[0, 0, 10, 10], [10, 0, 20, 10], [20, 10, 30, 20], [-50, -50, -40, -40]]])
    A = A.astype(np.int32)
    p, s, m = ctx.interactions(A)
    ep, es, em = oracle.interactions(A)
    assert (p, s) == (ep, es)
    assert np.array_equal(m, em)


def test_interactions_dense(ctx, oracle):
    L = stdcell_layers(30000, seed=9)
    for name in ("poly", "met1", "met2", "li1", "contact"):
        assert ctx.interactions(L[name])[:2] == oracle.interactions(L[name])[:2], name
    M = macro_arrays(nmacro=2, seed=10)
    assert ctx.interactions(M)[:2] == oracle.interactions(M)[:2]


def test_certify_healing(ctx, oracle):
    A = random_layer(20000, die=400_000, seed=11)
    assert not ctx.certify_healing(A)
    assert ctx.certify_healing(oracle.merge(A))
    assert ctx.certify_healing(A[:1]) and ctx.certify_healing(A[:0])
    p, s, m = ctx.interactions(A[:0])
    assert (p, s, len(m)) == (0, 0, 0)


@pytest.mark.parametrize("seed", [0, 1])
def test_component_areas(ctx, oracle, seed):
    A = random_layer(40000, die=700_000, seed=20 + seed)
    got = ctx.component_areas(A)
    exp = oracle.component_areas(A)
    assert np.array_equal(got, exp)
    assert got.sum() == oracle.union_area(A)


def test_component_areas_shapes(ctx, oracle):
    A = np.array([[0, 0, 10, 10], [5, 5, 15, 15], [20, 0, 30, 10], [30, 0, 40, 10], [100, 100, 110, 110]], np.int32)
    assert ctx.component_areas(A).tolist() == [100, 175, 200]
    assert ctx.component_areas(A[:0]).tolist() == [0]
    L = stdcell_layers(20000, seed=12)
    both = np.concatenate([L["met1"], L["met2"], L["contact"]])
    assert np.array_equal(ctx.component_areas(both), oracle.component_areas(both))
    M = macro_arrays(nmacro=2, seed=13)
    assert np.array_equal(ctx.component_areas(M), oracle.component_areas(M))


def test_deck_single_layer_and(tmp_path, monkeypatch, oracle):
    from vlsi_layout_gb300 import engine
    import test_gpu_deck as td
    monkeypatch.chdir(tmp_path)
    P = random_layer(6000, die=200_000, seed=14)
    td._write_mag(str(tmp_path / "d.mag"), {"poly": P})
    (tmp_path / "a.ctr").write_text("program a\ndecl design d1 = d.mag\ndecl output o1 = out.mag\n"
                                    "decl memory t1 = nothing\nexec init t1:nothing\n"
                                    "exec run o1:ov = d1:poly AND t1:nothing\n"
                                    "exec run t1:h = d1:poly + t1:nothing\n"
                                    "exec run t1:z = t1:h AND t1:nothing\n"
                                    "exec run t1:nothing = t1:z ASSERT_ZERO t1:nothing\nflush\nend\n")
    rc, log, fails = engine.run_deck(str(tmp_path / "a.ctr"))
    assert rc == 0 and fails == 0, log
    out = td._read_mag(str(tmp_path / "out.mag"))
    assert np.array_equal(td._canon(out["ov"]), oracle.overlap(P))
    (tmp_path / "g.ctr").write_text("program g\ndecl design d1 = d.mag\ndecl memory t1 = nothing\n"
                                    "exec init t1:nothing\nexec run t1:x = d1:poly GRID t1:nothing\nend\n")
    rc, log, fails = engine.run_deck(str(tmp_path / "g.ctr"))
    assert rc == engine.GB_ERR_ARG and "GRID" in log
