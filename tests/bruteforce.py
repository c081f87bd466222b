"""Independent brute-force restatement of the canonical strip form, for small
inputs only (pure numpy, O(n^2) cells): rasterise the Boolean of two box sets
on the compressed grid of all box coordinates and the 2^g tile lines, then
read off, per tile, the maximal y-runs of every x-slab and merge runs that
persist unchanged across consecutive x-slabs (the heal_boxes form)."""
import numpy as np


def _pred(op, ca, cb):
    """ca, cb: per-cell coverage counts of A and B."""
    if op == 7:  # single-layer AND: covered at least twice
        return ca >= 2
    a, b = ca > 0, cb > 0
    return [a ^ b, a | b, a & b, a & ~b, a][op]


def canonical(A, B, op, g=16):
    A = np.asarray(A, np.int64).reshape(-1, 4)
    B = np.asarray(B, np.int64).reshape(-1, 4)
    allb = np.concatenate([A, B]) if op not in (4, 7) else A
    if len(allb) == 0:
        return np.zeros((0, 4), np.int32)
    xs = set(allb[:, 0]) | set(allb[:, 2])
    ys = set(allb[:, 1]) | set(allb[:, 3])
    G = 1 << g
    for t in range(allb[:, 0].min() // G, allb[:, 2].max() // G + 1):
        xs.add(t * G)
    for t in range(allb[:, 1].min() // G, allb[:, 3].max() // G + 1):
        ys.add(t * G)
    xs = np.array(sorted(xs))
    ys = np.array(sorted(ys))
    cov = {}
    for name, S in (("a", A), ("b", B)):
        m = np.zeros((len(xs) - 1, len(ys) - 1), np.int32)
        for x1, y1, x2, y2 in S:
            i1, i2 = np.searchsorted(xs, x1), np.searchsorted(xs, x2)
            j1, j2 = np.searchsorted(ys, y1), np.searchsorted(ys, y2)
            m[i1:i2, j1:j2] += 1
        cov[name] = m
    R = _pred(op, cov["a"], cov["b"])
    out = []
    tx = xs[:-1] // G
    ty = ys[:-1] // G
    for tyv in np.unique(ty):
        jsel = np.where(ty == tyv)[0]
        for txv in np.unique(tx):
            isel = np.where(tx == txv)[0]
            open_runs = {}
            prev = set()
            for i in list(isel) + [None]:
                cur = set()
                if i is not None:
                    col = R[i, jsel]
                    j = 0
                    while j < len(jsel):
                        if col[j]:
                            k = j
                            while k + 1 < len(jsel) and col[k + 1]:
                                k += 1
                            cur.add((ys[jsel[j]], ys[jsel[k] + 1]))
                            j = k + 1
                        else:
                            j += 1
                xnow = xs[i] if i is not None else xs[isel[-1] + 1]
                for r in prev - cur:
                    out.append((open_runs.pop(r), r[0], xnow, r[1]))
                for r in cur - prev:
                    open_runs[r] = xnow
                prev = cur
    out = np.array(sorted(out), np.int64).reshape(-1, 4).astype(np.int32)
    return out
