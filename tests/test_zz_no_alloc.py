"""The no-allocation Boolean entry point (gb_bool_tile_noalloc).

Some callers cannot allocate device memory on their call path: a serving loop
that reserved its whole device budget up front, or a Fortran / C host that
owns only the buffers it passes.  This entry point works in storage the
library reserves statically.  These tests call it through the C-ABI with
device buffers and check it against the CPU oracle strip for strip, twice in a
row (the second call reuses the static storage the first one left behind),
and check every refusal: the status and *d_count == -1.  The file is named to
be collected last.
"""
import numpy as np
import pytest

from gen import random_layer

pytestmark = pytest.mark.gpu


def _canon(b):
    b = np.asarray(b, np.int32).reshape(-1, 4)
    return b[np.lexsort((b[:, 3], b[:, 2], b[:, 1], b[:, 0]))] if len(b) else b


def _noalloc(torch, engine, A, B, op, cap=65536):
    dA = torch.from_numpy(np.ascontiguousarray(A, np.int32).reshape(-1, 4)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B, np.int32).reshape(-1, 4)).cuda()
    out = torch.zeros((max(cap, 1), 4), dtype=torch.int32, device="cuda")
    cnt = torch.full((1,), 12345, dtype=torch.int64, device="cuda")   # stale values the call must overwrite
    area = torch.full((1,), 12345, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rc = engine.lib().gb_bool_tile_noalloc(op, dA.data_ptr(), len(dA), dB.data_ptr(), len(dB), out.data_ptr(), cap,
                                           cnt.data_ptr(), area.data_ptr(), None)
    n = int(cnt.item())
    return rc, n, (out[:n].cpu().numpy() if n >= 0 else None), int(area.item())


def test_noalloc_matches_oracle(oracle):
    torch = pytest.importorskip("torch")
    from vlsi_layout_gb300 import engine
    ox, oy = 3 * 65536, -2 * 65536
    A = random_layer(3000, die=65536, seed=31, x0=ox, y0=oy)
    B = random_layer(3000, die=65536, seed=32, x0=ox, y0=oy)
    for op in (engine.AND, engine.NOT, engine.OR, engine.XOR, engine.MERGE):
        ref = oracle.merge(A) if op == engine.MERGE else oracle.boolean(A, B, op)
        r64 = ref.astype(np.int64)
        ref_area = int(((r64[:, 2] - r64[:, 0]) * (r64[:, 3] - r64[:, 1])).sum())
        for _ in range(2):  # two calls in a row share the static storage
            rc, n, got, area = _noalloc(torch, engine, A, B, op)
            assert rc == engine.GB_OK and n == len(ref), (op, rc, n, len(ref))
            assert np.array_equal(_canon(got), ref), op
            assert area == ref_area


def test_noalloc_merge_ignores_b(oracle):
    """MERGE reads A only: a B outside A's tile is not refused."""
    torch = pytest.importorskip("torch")
    from vlsi_layout_gb300 import engine
    A = random_layer(800, die=65536, seed=35)
    far = np.array([[900000, 900000, 900010, 900010]], np.int32)
    rc, n, got, _ = _noalloc(torch, engine, A, far, engine.MERGE)
    assert rc == engine.GB_OK and np.array_equal(_canon(got), oracle.merge(A))


def test_noalloc_limits(oracle):
    torch = pytest.importorskip("torch")
    from vlsi_layout_gb300 import engine
    big = random_layer(16385, die=65536, seed=33)
    rc, n, got, area = _noalloc(torch, engine, big, big[:0], engine.MERGE)
    assert rc == engine.GB_ERR_CAPACITY and n == -1 and area == -1
    two_tiles = np.array([[0, 0, 10, 10], [70000, 0, 70010, 10]], np.int32)
    rc, n, got, area = _noalloc(torch, engine, two_tiles, two_tiles[:0], engine.MERGE)
    assert rc == engine.GB_ERR_INVALID_BOX and n == -1 and got is None
    # a result larger than the caller's buffer is a capacity error, not a silent empty result
    A = random_layer(500, die=65536, seed=34)
    ref = oracle.merge(A)
    rc, n, got, area = _noalloc(torch, engine, A, A[:0], engine.MERGE, cap=len(ref) - 1)
    assert rc == engine.GB_ERR_CAPACITY and n == -1 and area == -1
    # a valid call after the refusals still works, with a buffer of exactly the result's size
    rc, n, got, _ = _noalloc(torch, engine, A, A[:0], engine.MERGE, cap=len(ref))
    assert rc == engine.GB_OK and np.array_equal(_canon(got), ref)
