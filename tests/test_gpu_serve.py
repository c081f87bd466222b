"""Serving loop: requests on resident layers are admitted into concurrent
slots as they arrive; every result is the same alone and in the mix, and
matches the oracle."""
import numpy as np
import pytest

from gen import random_layer

pytestmark = pytest.mark.gpu


def _canon(b):
    return b[np.lexsort((b[:, 3], b[:, 2], b[:, 1], b[:, 0]))] if len(b) else b


def _requests(engine, rng, nl, n):
    ops = [0, 1, 2, 3, engine.REQ_SIZE, engine.REQ_GROW]
    r = np.zeros(n, engine.REQUEST_DTYPE)
    for i in range(n):
        op = ops[i % len(ops)]
        r[i]["op"] = op
        r[i]["a"] = rng.integers(0, nl)
        r[i]["b"] = rng.integers(0, nl)
        r[i]["amount"] = (-1 if i % 4 == 0 else 2) if op == engine.REQ_SIZE else 1
    return r


def _expected(oracle, engine, layers, q):
    A = layers[q["a"]]
    if q["op"] <= 3:
        return oracle.boolean(A, layers[q["b"]], int(q["op"]))
    if q["op"] == engine.REQ_SIZE:
        return oracle.size(A, int(q["amount"]))
    a = int(q["amount"])
    return oracle.grow(A, a, a, a, a)


def test_alone_and_in_the_mix(oracle):
    from vlsi_layout_gb300 import engine
    rng = np.random.default_rng(51)
    sizes = [1000, 3000, 8000, 20000, 50000, 2000]
    layers = [random_layer(n, die=int(1e6 * np.sqrt(n / 1e5)), seed=60 + i) for i, n in enumerate(sizes)]
    reqs = _requests(engine, rng, len(layers), 24)
    alone = []
    with engine.Server(budget_bytes=8 << 30, slots=1, slot_arena_bytes=2 << 30) as s1:
        ids = [s1.add_layer(L) for L in layers]
        assert ids == list(range(len(layers)))
        for i in range(len(reqs)):
            res = s1.run(reqs[i:i + 1], keep_outputs=True)
            assert res[0]["status"] == 0
            alone.append(_canon(s1.result_boxes(0)))
    with engine.Server(budget_bytes=8 << 30, slots=4, slot_arena_bytes=2 << 30) as s4:
        for L in layers:
            s4.add_layer(L)
        mix = reqs.copy()
        mix["arrival_s"] = np.sort(rng.exponential(1 / 2000.0, len(mix)).cumsum())  # Poisson, 2000 req/s
        res = s4.run(mix, keep_outputs=True)
        assert (res["status"] == 0).all()
        assert (res["latency_ms"] > 0).all() and (res["end_s"] >= res["start_s"]).all()
        for i in range(len(reqs)):
            got = _canon(s4.result_boxes(i))
            assert np.array_equal(got, alone[i]), i
            assert res[i]["count"] == len(got)
    for i in (0, 3, 4, 5, 10):
        assert np.array_equal(alone[i], _expected(oracle, engine, layers, reqs[i])), i


def test_budget_admission():
    from vlsi_layout_gb300 import engine
    with engine.Server(budget_bytes=2 << 20, slots=2, slot_arena_bytes=1 << 30) as s:
        a = s.add_layer(random_layer(100000, seed=70))
        r = np.zeros(1, engine.REQUEST_DTYPE)
        r[0]["op"], r[0]["a"], r[0]["b"] = 2, a, a
        res = s.run(r)
        assert res[0]["status"] == engine.GB_ERR_CAPACITY  # can never fit the 2 MiB budget
