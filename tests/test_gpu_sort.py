"""Device radix sort (the Morton / event-key sort of gpu_morton.cu:149-187 and
event_sorter.cu:64-81) against a stable numpy sort of the same keys: every
built configuration (pass count x tile size), ragged sizes around the
tile edges, unaligned buffers (plain-load path), skewed digit distributions,
Morton keys of real box shapes, and the autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def expect(keys, vals, bits):
    m = np.uint64((1 << bits) - 1) if bits < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    o = np.argsort(keys & m, kind="stable")
    return keys[o], vals[o]


def dev_sort(ctx, keys, vals, bits, passes=0, tile=0, offset=0):
    """Sort on the device; offset > 0 shifts the buffers by that many elements
    so they are not 16-byte aligned."""
    n = len(keys)
    kb = torch.zeros(n + offset, dtype=torch.int64, device="cuda")
    vb = torch.zeros(n + offset, dtype=torch.int32, device="cuda")
    kt = torch.zeros(n + offset, dtype=torch.int64, device="cuda")
    vt = torch.zeros(n + offset, dtype=torch.int32, device="cuda")
    kb[offset:] = torch.from_numpy(keys.view(np.int64)).cuda()
    vb[offset:] = torch.from_numpy(vals.view(np.int32)).cuda()
    torch.cuda.synchronize()
    k, v = kb[offset:], vb[offset:]
    p = ctx.radix_sort_device(k.data_ptr(), v.data_ptr(), n, bits, kt[offset:].data_ptr(), vt[offset:].data_ptr(),
                              passes, tile)
    ctx.sync()
    return k.cpu().numpy().view(np.uint64), v.cpu().numpy().view(np.uint32), p


def rand_keys(n, bits, seed):
    r = np.random.default_rng(seed)
    k = r.integers(0, 1 << min(bits, 63), size=n, dtype=np.uint64)
    if bits == 64:
        k |= r.integers(0, 2, size=n, dtype=np.uint64) << np.uint64(63)
    return k, np.arange(n, dtype=np.uint32)


@pytest.mark.parametrize("tile", [3072, 4096, 5120, 6144, 8192])
@pytest.mark.parametrize("bits,passes", [(8, 1), (20, 2), (20, 3), (40, 4), (40, 5), (40, 6), (52, 6), (52, 7),
                                         (52, 8), (64, 7), (64, 8)])
def test_configs(ctx, tile, bits, passes):
    keys, vals = rand_keys(300_007, bits, seed=bits * 31 + passes)
    k, v, p = dev_sort(ctx, keys, vals, bits, passes, tile)
    ek, ev = expect(keys, vals, bits)
    assert p == passes
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


@pytest.mark.parametrize("n", [2, 3, 5, 31, 1000, 4095, 4096, 4097, 5121, 65537, 1 << 20])
def test_ragged_sizes(ctx, n):
    keys, vals = rand_keys(n, 40, seed=n)
    k, v, _ = dev_sort(ctx, keys, vals, 40)
    ek, ev = expect(keys, vals, 40)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


@pytest.mark.parametrize("offset", [1, 3])
def test_unaligned_buffers(ctx, offset):
    keys, vals = rand_keys(200_003, 52, seed=7 + offset)
    k, v, _ = dev_sort(ctx, keys, vals, 52, offset=offset)
    ek, ev = expect(keys, vals, 52)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


def test_skewed_digits(ctx):
    r = np.random.default_rng(3)
    n = 500_000
    cases = {
        "all_equal": np.full(n, 0x123456789, np.uint64),
        "few_distinct": r.choice(np.array([5, 1 << 30, 7 << 20, 0], np.uint64), n),
        "constant_high": (np.uint64(0xABC) << np.uint64(40)) | r.integers(0, 1 << 12, n, dtype=np.uint64),
        "descending": np.arange(n, 0, -1, dtype=np.uint64) << np.uint64(9),
    }
    vals = np.arange(n, dtype=np.uint32)
    for name, keys in cases.items():
        for bits in (44, 52):
            k, v, _ = dev_sort(ctx, keys, vals, bits)
            ek, ev = expect(keys, vals, bits)
            assert np.array_equal(k, ek) and np.array_equal(v, ev), (name, bits)


def test_high_bits_ignored(ctx):
    """Keys are ordered by their low `bits` bits only; the rest ride along."""
    keys, vals = rand_keys(100_000, 64, seed=11)
    k, v, _ = dev_sort(ctx, keys, vals, 24)
    ek, ev = expect(keys, vals, 24)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


def test_morton_keys_of_boxes(ctx, oracle):
    from gen import random_layer
    boxes = random_layer(400_000, die=40_000_000, seed=5)
    keys = oracle.morton_keys_np(boxes)
    span = int((keys ^ keys[0]).max())
    bits = max(1, span.bit_length())
    vals = np.arange(len(keys), dtype=np.uint32)
    k, v, _ = dev_sort(ctx, keys, vals, bits)
    ek, ev = expect(keys, vals, bits)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


def test_bad_configuration(ctx):
    from vlsi_layout_gb300 import engine
    keys, vals = rand_keys(1000, 40, seed=1)
    with pytest.raises(engine.GBError):
        dev_sort(ctx, keys, vals, 40, passes=2, tile=4096)  # 20-bit digits are not built
    with pytest.raises(engine.GBError):
        dev_sort(ctx, keys, vals, 40, passes=5, tile=1000)  # no kernel has 1000-key tiles


def test_autotune(ctx):
    from vlsi_layout_gb300 import engine
    n, bits = 2_000_000, 48
    keys, vals = rand_keys(n, bits, seed=9)
    kd = torch.from_numpy(keys.view(np.int64)).cuda()
    vd = torch.from_numpy(vals.view(np.int32)).cuda()
    torch.cuda.synchronize()
    try:
        p, it, ms = ctx.radix_autotune(kd.data_ptr(), vd.data_ptr(), n, bits)
        assert 1 <= p <= bits and it in (3072, 4096, 5120, 6144, 8192) and ms > 0
        # the inputs are untouched, and the default sort now runs the tuned configuration
        assert np.array_equal(kd.cpu().numpy().view(np.uint64), keys)
        k, v, pp = dev_sort(ctx, keys, vals, bits)
        assert pp == p
        ek, ev = expect(keys, vals, bits)
        assert np.array_equal(k, ek) and np.array_equal(v, ev)
    finally:
        engine.lib().gb_radix_tuning_reset()
