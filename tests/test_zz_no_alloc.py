"""The no-allocation Boolean entry point (gb_bool_tile_noalloc).

Some callers cannot allocate device memory on their call path (a serving loop
that reserved its whole device budget up front, or a host that owns only the
buffers it passes).  This entry point works in storage the library reserves
statically; these tests call it through the C-ABI with device buffers and
check it against the layer API (gb_op_bool) bit for bit, twice in a row, so a
second call that reuses the static storage must give the same result.  The
file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from gen import random_layer

pytestmark = pytest.mark.gpu


def _canon(b):
    b = np.asarray(b, np.int32).reshape(-1, 4)
    return b[np.lexsort((b[:, 3], b[:, 2], b[:, 1], b[:, 0]))] if len(b) else b


def _noalloc(torch, engine, A, B, op, cap=65536):
    dA = torch.from_numpy(np.ascontiguousarray(A, np.int32)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B, np.int32)).cuda()
    out = torch.zeros((cap, 4), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    area = torch.zeros(1, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rc = engine.lib().gb_bool_tile_noalloc(op, dA.data_ptr(), len(A), dB.data_ptr(), len(B), out.data_ptr(), cap,
                                           cnt.data_ptr(), area.data_ptr(), None)
    n = int(cnt.item())
    return rc, (out[:max(n, 0)].cpu().numpy() if n >= 0 else None), int(area.item())


def test_noalloc_matches_layer_api():
    torch = pytest.importorskip("torch")
    from vlsi_layout_gb300 import engine
    ox, oy = 3 * 65536, -2 * 65536
    A = random_layer(3000, die=65536, seed=31, x0=ox, y0=oy)
    B = random_layer(3000, die=65536, seed=32, x0=ox, y0=oy)
    with engine.Context(0) as ctx:
        for op in (engine.AND, engine.NOT, engine.OR, engine.XOR, engine.MERGE):
            m = ctx.mark()
            LA, LB = ctx.layer(A), ctx.layer(B)
            ref = _canon(ctx.op(op, LA, LB).to_numpy())
            ctx.release(m)
            for _ in range(2):  # two calls in a row share the static storage
                rc, got, area = _noalloc(torch, engine, A, B, op)
                assert rc == engine.GB_OK
                assert np.array_equal(_canon(got), ref), op
                r64 = ref.astype(np.int64)
                assert area == int(((r64[:, 2] - r64[:, 0]) * (r64[:, 3] - r64[:, 1])).sum())


def test_noalloc_limits():
    torch = pytest.importorskip("torch")
    from vlsi_layout_gb300 import engine
    big = random_layer(16385, die=65536, seed=33)
    rc, got, _ = _noalloc(torch, engine, big, big[:0], engine.MERGE)
    assert rc == engine.GB_ERR_CAPACITY
    two_tiles = np.array([[0, 0, 10, 10], [70000, 0, 70010, 10]], np.int32)
    rc, got, _ = _noalloc(torch, engine, two_tiles, two_tiles[:0], engine.MERGE)
    assert rc == engine.GB_ERR_INVALID_BOX and got is None
    # a valid call after the refusals still works
    A = random_layer(500, die=65536, seed=34)
    rc, got, _ = _noalloc(torch, engine, A, A[:0], engine.MERGE)
    assert rc == engine.GB_OK and len(got) > 0
