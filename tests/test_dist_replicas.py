"""The multi-rank (replica) logic of bench.py on CPU: two gloo ranks on
127.0.0.1 agree on the slowest rank's time, report the whole-job value, and
only rank 0 runs and prints the reference arm."""
import contextlib
import io
import json
import os
import socket
import sys
import types

import pytest

torch = pytest.importorskip("torch")
mp = torch.multiprocessing

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, dist = bench.dist_init()
    ms = bench.max_over_ranks(dist, 10.0 + 5.0 * r)  # rank 1 is the slow one
    value = bench.replica_value(w, 1000, ms)
    boxes, off = bench.make_cells(6, median=300, seed=1)
    args = types.SimpleNamespace(steps=1, warmup=0, ref_boxes=500)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(args, boxes, off, w, r, dist)
    dist.barrier()
    dist.destroy_process_group()
    q.put((r, w, ms, value, buf.getvalue()))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, ms0, v0, out0), (r1, w1, ms1, v1, out1) = res
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert ms0 == ms1 == 15.0  # both ranks report the slowest rank's time
    assert v0 == v1 == 2 * 1000 / 0.015  # whole-job throughput over both replicas
    line = json.loads(out0.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert out1 == ""  # the other ranks exit without work
