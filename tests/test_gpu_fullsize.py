"""The workloads at their full sizes.

Oracle parity: the standard-cell layout at its full size (four layers of 10M
boxes: AND / NOT / OR / XOR of poly x li1, met1 x met2 and li1 x met1, and the
PNUM labels of met1 + met2 through the 2% contacts) against the CPU oracle on
all host cores, strip digests and counts per result, labels bit for bit; and
a 4e6 x 4e6-dbu window of the full-chip layer (clipped standard-cell boxes and
macro arrays) through the whole OP1 deck, every layer's strips against the
oracle's.

Properties of the whole 360M-box full-chip layer (where an oracle run of the
deck would take too long): the Morton sort's order and permutation, the OP1
ASSERT_ZEROs, additivity of area over a partition, invariance of the component
count under box order, and agreement of two kernels on the singletons; and
point-set identities of the standard-cell Booleans."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev_layer(ctx, t, off=None):
    from vlsi_layout_gb300 import engine
    h = ctypes.c_void_p()
    ncell = 1 if off is None else off.shape[0] - 1
    torch.cuda.synchronize()
    ctx._chk(engine.lib().gb_layer_from_device(ctx.h, t.data_ptr(), t.shape[0],
                                               None if off is None else off.data_ptr(), ncell,
                                               ctypes.byref(h)))
    return engine.Layer(ctx, h, ncell)


def area(ctx, L):
    return ctx.area(L)


@pytest.fixture(scope="module")
def std10m():
    from gen_device import stdcell_layers
    L = stdcell_layers(10_000_000, die=6_700_000, seed=1)
    torch.cuda.synchronize()
    yield L
    del L
    torch.cuda.empty_cache()


def test_stdcell_10m_boolean_identities(ctx, std10m):
    from vlsi_layout_gb300 import engine as E
    for a, b in (("poly", "li1"), ("met1", "met2"), ("li1", "met1")):
        m = ctx.mark()
        try:
            A, B = dev_layer(ctx, std10m[a]), dev_layer(ctx, std10m[b])
            aa, bb = int(area(ctx, A)[0]), int(area(ctx, B)[0])
            u = int(area(ctx, ctx.op(E.OR, A, B))[0])
            i = int(area(ctx, ctx.op(E.AND, A, B))[0])
            d = int(area(ctx, ctx.op(E.NOT, A, B))[0])
            x = int(area(ctx, ctx.op(E.XOR, A, B))[0])
            assert u + i == aa + bb and d + i == aa and x == u - i, (a, b)
            assert i > 0 and d > 0
            assert ctx.op(E.XOR, A, A).count()[0] == 0
            # a healed layer has no area covered twice, the raw one has
            assert ctx.op(E.OVERLAP, ctx.op(E.MERGE, A)).count()[0] == 0
        finally:
            ctx.release(m)


def test_stdcell_10m_connectivity(ctx, std10m):
    both = torch.cat([std10m["met1"], std10m["met2"], std10m["contact"]]).cpu().numpy()
    n1, lab = ctx.components(both)
    perm = np.random.default_rng(0).permutation(len(both))
    n2, lab2 = ctx.components(both[perm])
    assert n1 == n2
    # the same partition: label pairs (old, new) are a bijection, singletons stay 0
    lp = lab[perm]
    assert np.array_equal(lp == 0, lab2 == 0)
    code = np.unique(lp * (int(lab2.max()) + 1) + lab2)
    assert len(code) == len(np.unique(lab2))
    # singletons of the union-find agree with the pair-statistics kernel
    p, s, mask = ctx.interactions(both)
    assert s == int((lab == 0).sum()) and np.array_equal(mask.astype(bool), lab == 0)
    assert p > 0


@pytest.fixture(scope="module")
def std10m_host():
    from gen import stdcell_layers
    return stdcell_layers(10_000_000, die=6_700_000, seed=1)


def test_stdcell_10m_oracle_parity(ctx, oracle, std10m_host):
    """Standard-cell workload at 10M boxes per layer: every pairwise Boolean's
    strips (per-layer digest and count) equal the oracle's."""
    from vlsi_layout_gb300 import engine as E
    L = std10m_host
    for a, b in (("poly", "li1"), ("met1", "met2"), ("li1", "met1")):
        m = ctx.mark()
        try:
            A, B = ctx.layer(L[a]), ctx.layer(L[b])
            for op in (E.AND, E.NOT, E.OR, E.XOR):
                R = ctx.op(op, A, B)
                e = oracle.boolean(L[a], L[b], op)
                assert R.count()[0] == len(e), (a, b, op)
                assert int(R.digest()[0]) == oracle.strip_digest(e), (a, b, op)
                if op == E.AND and a == "met1":  # one result strip for strip
                    assert np.array_equal(oracle.canonical(R.to_numpy()), e)
        finally:
            ctx.release(m)


def test_stdcell_10m_components_oracle(ctx, oracle, std10m_host):
    """PNUM labels of met1 + met2 joined through the 2% contacts, bit for bit
    against the oracle's union-find (closed overlap, min-index roots)."""
    L = std10m_host
    both = np.concatenate([L["met1"], L["met2"], L["contact"]])
    n, lab = ctx.components(both)
    en, elab = oracle.components(both)
    assert n == en and np.array_equal(lab, elab)


@pytest.fixture(scope="module")
def chip():
    from gen_device import full_chip
    t = full_chip(360_000_000, 40_000_000, seed=3)
    torch.cuda.synchronize()
    yield t
    del t
    torch.cuda.empty_cache()


def test_full_chip_morton_sort(ctx, chip):
    from vlsi_layout_gb300 import engine
    L = engine.lib()
    n = chip.shape[0]
    keys = torch.empty(n, dtype=torch.int64, device="cuda")
    vals = torch.empty(n, dtype=torch.int32, device="cuda")
    kt, vt = torch.empty_like(keys), torch.empty_like(vals)
    torch.cuda.synchronize()
    L.gb_morton_keys_device(ctx.h, chip.data_ptr(), n, keys.data_ptr(), vals.data_ptr())
    ctx.sync()
    bits = max(1, int((keys ^ keys[0]).max().item()).bit_length())
    assert bits <= 64
    ctx.radix_sort_device(keys.data_ptr(), vals.data_ptr(), n, bits, kt.data_ptr(), vt.data_ptr())
    ctx.sync()
    del kt, vt
    # bits above `bits` are the same in every key, so signed order is key order
    assert bool((keys[1:] >= keys[:-1]).all().item())
    v = vals.long()
    cnt = torch.bincount(v, minlength=n)
    assert int(cnt.min().item()) == 1 and int(cnt.max().item()) == 1
    del cnt
    g = chip[v].contiguous()
    del v
    k2 = torch.empty_like(keys)
    v2 = torch.empty_like(vals)
    torch.cuda.synchronize()
    L.gb_morton_keys_device(ctx.h, g.data_ptr(), n, k2.data_ptr(), v2.data_ptr())
    ctx.sync()
    assert torch.equal(k2, keys)


def test_full_chip_op1_and_area(ctx, chip):
    m = ctx.mark()
    try:
        P = dev_layer(ctx, chip)
        outs = ctx.op1(P, 1)
        assert outs[4].count()[0] == 0 and outs[5].count()[0] == 0  # the two ASSERT_ZEROs
        a = int(area(ctx, P)[0])
        assert int(area(ctx, outs[0])[0]) > a > int(area(ctx, outs[1])[0])
    finally:
        ctx.release(m)
    # additivity over a partition: four quadrant cells of clipped boxes
    half = 20_000_000
    parts, offs = [], [0]
    for qx, qy in ((0, 0), (1, 0), (0, 1), (1, 1)):
        x0, y0 = qx * half, qy * half
        c = chip.clone()
        c[:, 0].clamp_(min=x0)
        c[:, 1].clamp_(min=y0)
        c[:, 2].clamp_(max=x0 + half)
        c[:, 3].clamp_(max=y0 + half)
        c = c[(c[:, 0] < c[:, 2]) & (c[:, 1] < c[:, 3])]
        parts.append(c)
        offs.append(offs[-1] + c.shape[0])
    cat = torch.cat(parts).contiguous()
    del parts
    off = torch.tensor(offs, dtype=torch.int64, device="cuda")
    m = ctx.mark()
    try:
        Q = dev_layer(ctx, cat, off)
        assert int(area(ctx, Q).sum()) == a
    finally:
        ctx.release(m)


def test_full_chip_window_oracle(ctx, oracle, chip):
    """A 4e6 x 4e6-dbu window of the full-chip layer (boxes clipped to it:
    standard-cell shapes and a few hundred 64x64 macro arrays) through the OP1
    deck: every result layer's strips equal the oracle's (digest and count),
    MERGE strip for strip, and the union area."""
    from vlsi_layout_gb300 import engine as E
    x0, y0, w = 8_000_000, 12_000_000, 4_000_000
    c = chip[(chip[:, 2] > x0) & (chip[:, 0] < x0 + w) & (chip[:, 3] > y0) & (chip[:, 1] < y0 + w)].clone()
    c[:, 0].clamp_(min=x0)
    c[:, 1].clamp_(min=y0)
    c[:, 2].clamp_(max=x0 + w)
    c[:, 3].clamp_(max=y0 + w)
    win = c.cpu().numpy()
    nmacro_boxes = int(((win[:, 2] - win[:, 0] == 200) & (win[:, 3] - win[:, 1] == 200)).sum())
    assert len(win) > 2_000_000 and nmacro_boxes > 100_000
    ec, ea, ed = oracle.op1_digest(win, 1)
    m = ctx.mark()
    try:
        P = ctx.layer(win)
        outs = ctx.op1(P, 1)
        for j, L in enumerate(outs):
            assert L.count()[0] == ec[j], j
            assert int(L.digest()[0]) == int(ed[j]), j
        M = ctx.op(E.MERGE, P)
        assert int(M.digest()[0]) == int(ed[6])
        assert np.array_equal(oracle.canonical(M.to_numpy()), oracle.merge(win))
        assert int(ctx.area(P)[0]) == ea
    finally:
        ctx.release(m)


def test_full_chip_components(ctx, chip):
    host = chip.cpu().numpy()
    n1, lab = ctx.components(host)
    perm = torch.randperm(host.shape[0], generator=torch.Generator().manual_seed(5)).numpy()
    n2, lab2 = ctx.components(host[perm])
    assert n1 == n2
    assert int((lab == 0).sum()) == int((lab2 == 0).sum())
    p, s, mask = ctx.interactions(host)
    assert s == int((lab == 0).sum())
    assert p > 0
