"""GPU parity on tile grids other than 2^16 (the slab height the autotuner
picks): every operator bit-exact to the oracle at the same grid, results
carried across a grid change, and the tuner's choice."""
import numpy as np
import pytest

from gen import cells_layout, random_layer

pytestmark = pytest.mark.gpu


def canon(b):
    b = np.asarray(b, np.int32).reshape(-1, 4)
    return b[np.lexsort((b[:, 3], b[:, 2], b[:, 1], b[:, 0]))] if len(b) else b


@pytest.fixture
def grid_ctx(ctx):
    yield ctx
    ctx.set_grid(16)


@pytest.mark.parametrize("g", [13, 14, 15])
def test_ops_on_grid(grid_ctx, oracle, g):
    ctx = grid_ctx
    A = random_layer(20000, die=400000, seed=3, x0=-200000, y0=-70000)
    B = random_layer(20000, die=400000, seed=4, x0=-200000, y0=-70000)
    ctx.set_grid(g)
    assert ctx.grid == g
    m = ctx.mark()
    try:
        LA, LB = ctx.layer(A), ctx.layer(B)
        for op in (0, 1, 2, 3):
            got = canon(ctx.op(op, LA, LB).to_numpy())
            assert np.array_equal(got, oracle.boolean(A, B, op, grid_log2=g)), op
        assert np.array_equal(canon(ctx.op(4, LA).to_numpy()), oracle.merge(A, grid_log2=g))
        assert np.array_equal(canon(ctx.grow(LA, 3, 1, 2, 5).to_numpy()), oracle.grow(A, 3, 1, 2, 5, grid_log2=g))
        assert np.array_equal(canon(ctx.size(LA, -2).to_numpy()), oracle.size(A, -2, grid_log2=g))
        assert int(ctx.area(LA)[0]) == oracle.union_area(A)
    finally:
        ctx.release(m)


def test_result_carried_across_grids(grid_ctx, oracle):
    ctx = grid_ctx
    A = random_layer(8000, die=300000, seed=5)
    B = random_layer(8000, die=300000, seed=6)
    m = ctx.mark()
    try:
        LA, LB = ctx.layer(A), ctx.layer(B)
        ctx.set_grid(16)
        U = ctx.op(1, LA, LB)          # binned on 2^16 tiles
        ctx.set_grid(14)
        X = ctx.op(0, U, LA)           # re-binned on 2^14 tiles
        u16 = oracle.boolean(A, B, 1, grid_log2=16)
        assert np.array_equal(canon(X.to_numpy()), oracle.boolean(u16, A, 0, grid_log2=14))
    finally:
        ctx.release(m)


def test_grid_autotune(grid_ctx, oracle):
    ctx = grid_ctx
    boxes, off = cells_layout(32, median=3000, seed=8)
    m = ctx.mark()
    try:
        P = ctx.layer(boxes, off)
        g, ms = ctx.grid_autotune(P, 1)
        assert 13 <= g <= 16 and ctx.grid == g
        assert ms[g] is not None and all(v is None or v >= ms[g] for v in ms.values())
        outs = ctx.op1(P, 1)
        counts = np.stack([L.count()[1] for L in outs], axis=1)
        ec, ea = oracle.op1_cells(boxes, off, 1, grid_log2=g)
        assert np.array_equal(counts, ec)
    finally:
        ctx.release(m)
