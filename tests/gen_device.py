"""Seeded synthetic layouts generated on the GPU with torch, for the
full-size property tests (tens to hundreds of millions of boxes, where numpy
generation and an oracle run would take too long).  Shapes follow the
standard-cell and full-chip workloads: rows 2720 dbu tall, poly stripes 150
wide on 340-pitch tracks, met1/met2 wires 140 wide with lognormal(7, 1)
lengths, li1 rects 170..800, 2% contacts 170x170; macros are 64x64 arrays of
200x200 boxes at 400 pitch."""
import torch


def _gen(seed):
    return torch.Generator(device="cuda").manual_seed(seed)


def _ri(lo, hi, n, g):
    """uniform int64 in [lo, hi) (hi may be a tensor)."""
    if torch.is_tensor(hi):
        u = torch.rand(n, device="cuda", generator=g, dtype=torch.float64)
        return lo + (u * (hi - lo).to(torch.float64)).to(torch.int64)
    return torch.randint(lo, hi, (n,), device="cuda", generator=g, dtype=torch.int64)


def _lognormal_len(n, die, g):
    z = torch.randn(n, device="cuda", generator=g, dtype=torch.float64)
    return torch.clamp(torch.round(torch.exp(7.0 + z)), 140, die // 2).to(torch.int64)


def stdcell_layers(n, die, seed):
    """dict of int32 [n, 4] CUDA tensors: poly, met1, met2, li1 (n boxes each)
    and contact (n // 50)."""
    g = _gen(seed)
    px = _ri(0, die // 340, n, g) * 340
    py = _ri(0, die - 2600, n, g)
    pl = _ri(500, 2501, n, g)
    poly = torch.stack([px, py, px + 150, py + pl], 1)
    L = _lognormal_len(n, die, g)
    mx = _ri(0, die - L, n, g)
    my = _ri(0, die // 340, n, g) * 340
    met1 = torch.stack([mx, my, mx + L, my + 140], 1)
    L2 = _lognormal_len(n, die, g)
    nx = _ri(0, die // 340, n, g) * 340 + 100
    ny = _ri(0, die - L2, n, g)
    met2 = torch.stack([nx, ny, nx + 140, ny + L2], 1)
    w = _ri(170, 801, n, g)
    h = _ri(170, 801, n, g)
    lx = _ri(0, die - w, n, g)
    ly = _ri(0, die - h, n, g)
    li1 = torch.stack([lx, ly, lx + w, ly + h], 1)
    nc = max(1, n // 50)
    cx = _ri(0, die - 170, nc, g)
    cy = _ri(0, die - 170, nc, g)
    cont = torch.stack([cx, cy, cx + 170, cy + 170], 1)
    return {k: v.to(torch.int32).contiguous() for k, v in
            dict(poly=poly, met1=met1, met2=met2, li1=li1, contact=cont).items()}


def full_chip(n_total, die, seed, macro_frac=0.3):
    """One int32 [~n_total, 4] CUDA layer: standard-cell boxes (the four shapes
    mixed) over the die plus macros (64x64 arrays of 200x200 boxes at 400
    pitch) on distinct 26000-dbu slots."""
    g = _gen(seed)
    side, pitch, size = 64, 400, 200
    per_macro = side * side
    nmac = int(n_total * macro_frac) // per_macro
    slot = 26000
    nslot = die // slot
    pick = torch.randperm(nslot * nslot, device="cuda", generator=g)[:nmac]
    ox = (pick % nslot) * slot
    oy = (pick // nslot) * slot
    ii = torch.arange(side, device="cuda", dtype=torch.int64)
    gx = (ii.view(1, side, 1) * pitch).expand(1, side, side).reshape(1, -1)
    gy = (ii.view(1, 1, side) * pitch).expand(1, side, side).reshape(1, -1)
    mx = (ox.view(-1, 1) + gx).reshape(-1)
    my = (oy.view(-1, 1) + gy).reshape(-1)
    macros = torch.stack([mx, my, mx + size, my + size], 1)
    nstd = n_total - macros.shape[0]
    q = nstd // 4
    parts = stdcell_layers(q, die, seed + 1)
    std = torch.cat([parts["poly"], parts["met1"], parts["met2"], parts["li1"][: nstd - 3 * q]])
    out = torch.cat([std.to(torch.int64), macros]).to(torch.int32).contiguous()
    return out
