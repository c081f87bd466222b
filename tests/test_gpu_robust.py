"""Dense layouts (standard-cell rows, macro arrays, heavily overlapping
stacks that overflow the shared-memory buffers into scratch) against the
oracle, and the failure paths: bounded waits that time out, capacities that
are too small, invalid boxes.  No test faults the GPU: every failure is made
on the host side or by a bounded wait that nothing releases."""
import numpy as np
import pytest

from gen import macro_arrays, random_layer, stdcell_layers

pytestmark = pytest.mark.gpu


def canon(b):
    b = np.asarray(b, np.int32).reshape(-1, 4)
    return b[np.lexsort((b[:, 3], b[:, 2], b[:, 1], b[:, 0]))] if len(b) else b


def run(ctx, fn):
    m = ctx.mark()
    try:
        return canon(fn().to_numpy())
    finally:
        ctx.release(m)


def test_stdcell_layers(ctx, oracle):
    L = stdcell_layers(20000, seed=1)
    for a, b in (("poly", "li1"), ("met1", "met2"), ("met1", "contact")):
        for op in (0, 1, 2, 3):
            got = run(ctx, lambda: ctx.op(op, ctx.layer(L[a]), ctx.layer(L[b])))
            assert np.array_equal(got, oracle.boolean(L[a], L[b], op)), (a, b, op)
    got = run(ctx, lambda: ctx.size(ctx.layer(L["met1"]), -30))
    assert np.array_equal(got, oracle.size(L["met1"], -30))
    got = run(ctx, lambda: ctx.grow(ctx.layer(L["poly"]), 70, 0, 70, 0))
    assert np.array_equal(got, oracle.grow(L["poly"], 70, 0, 70, 0))
    n, lab = ctx.components(np.concatenate([L["met1"], L["met2"], L["contact"]]))
    en, elab = oracle.components(np.concatenate([L["met1"], L["met2"], L["contact"]]))
    assert n == en and np.array_equal(lab, elab)


def test_macro_arrays(ctx, oracle):
    M = macro_arrays(4)
    G = random_layer(3000, die=400000, seed=81)
    for op in (0, 2, 3, 4):
        got = run(ctx, lambda: ctx.op(op, ctx.layer(M), ctx.layer(G)) if op != 4 else ctx.op(4, ctx.layer(M)))
        exp = oracle.boolean(M, G, op) if op != 4 else oracle.merge(M)
        assert np.array_equal(got, exp), op
    got = run(ctx, lambda: ctx.size(ctx.layer(M), 100))  # dilation merges the array rows
    assert np.array_equal(got, oracle.size(M, 100))


def test_overflow_paths(ctx, oracle):
    # thousands of heavily overlapping boxes in one tile: local columns, local
    # values and the member bitmap all exceed their shared-memory buffers
    A = random_layer(20000, die=20000, wmin=20, wmax=3000, seed=82)
    B = random_layer(20000, die=20000, wmin=20, wmax=3000, seed=83)
    for op in (0, 3, 4):
        got = run(ctx, lambda: ctx.op(op, ctx.layer(A), ctx.layer(B)) if op != 4 else ctx.op(4, ctx.layer(A)))
        exp = oracle.boolean(A, B, op) if op != 4 else oracle.merge(A)
        assert np.array_equal(got, exp), op


def test_bounded_lookback_times_out(ctx):
    from vlsi_layout_gb300 import engine
    assert engine.lib().gb_debug_lookback_timeout(ctx.h, 1000) == engine.GB_ERR_TIMEOUT
    ctx.sync()  # the context is usable afterwards


def test_tiny_scratch_spills_and_stays_exact(oracle):
    # a 64 KiB per-CTA scratch forces every tile's buffers to spill into the
    # work arena; results must not change
    from vlsi_layout_gb300 import engine
    A = random_layer(20000, die=30000, seed=84)
    B = random_layer(20000, die=30000, seed=86)
    with engine.Context(0) as c:
        assert engine.lib().gb_set_tile_scratch(c.h, 1 << 16) == 0
        m = c.mark()
        got = canon(c.op(3, c.layer(A), c.layer(B)).to_numpy())
        assert np.array_equal(got, oracle.boolean(A, B, 3))
        c.release(m)
        counts, area, fails = c.op1_host(A.ctypes.data, len(A), np.array([0, len(A)]), 1)
        exp, earea = oracle.op1(A, 1)
        assert counts[0].tolist() == [exp[k] for k in ("poly_1", "poly_2", "outer_ring", "inner_ring",
                                                       "ring_and1", "ring_intersection")]
        assert int(area[0]) == earea and fails == 0


def test_small_arena_is_an_error():
    from vlsi_layout_gb300 import engine
    A = random_layer(100000, seed=85)
    with engine.Context(0, arena_bytes=1 << 20) as c:
        with pytest.raises(engine.GBError) as ei:
            c.op(4, c.layer(A)).to_numpy()
        assert ei.value.code == engine.GB_ERR_CAPACITY
        c.sync()


def test_invalid_boxes_are_rejected(ctx):
    from vlsi_layout_gb300 import engine
    bad = np.array([[0, 0, 10, 10], [5, 5, 5, 9]], np.int32)  # zero width
    m = ctx.mark()
    with pytest.raises(engine.GBError) as ei:
        ctx.op(4, ctx.layer(bad)).to_numpy()
    assert ei.value.code == engine.GB_ERR_INVALID_BOX
    ctx.release(m)
    ctx.sync()


def test_set_stream_leaves_caller_stream_alive():
    """A context that adopted the caller's stream must not destroy it on close."""
    torch = pytest.importorskip("torch")
    from vlsi_layout_gb300 import engine
    s = torch.cuda.Stream()
    c = engine.Context(0)
    c.set_stream(s.cuda_stream)
    m = c.mark()
    L = c.layer(random_layer(2000, die=50_000, seed=3))
    assert c.op(engine.MERGE, L).count()[0] > 0
    c.release(m)
    c.close()
    with torch.cuda.stream(s):
        x = torch.arange(1000, device="cuda") * 2
    s.synchronize()
    assert int(x.sum().item()) == 999000
