"""CPU tests of the SNAP host entry points that touch no GPU: the .snap header
reader (gb_snap_file_info) on files the oracle writes (serialization.f90
layout), empty and truncated files, and the stream bound of
gb_snap_max_bytes against the oracle's streams."""
import numpy as np
import pytest

import snapcases as S


def _lib():
    from vlsi_layout_gb300 import build as B
    B.build()
    from vlsi_layout_gb300 import engine
    return engine


def test_file_info(oracle, tmp_path):
    engine = _lib()
    A = S.cases()["chunk_plus_one"]
    pn = np.arange(len(A), dtype=np.int64)
    for method, props, pnum in ((1, 1, pn), (0, 32, None)):
        p = tmp_path / ("f%d.snap" % method)
        p.write_bytes(oracle.snap_file_bytes(A, method, props | (4 if pnum is not None else 0), pnum))
        n, nch, m, pr = engine.snap_file_info(str(p))
        assert (n, nch, m) == (len(A), 2, method)
        assert pr == props | (4 if pnum is not None else 0)
    e = tmp_path / "empty.snap"
    e.write_bytes(b"")
    assert engine.snap_file_info(str(e)) == (0, 0, 0, 0)


def test_file_info_rejects_truncated_files(oracle, tmp_path):
    engine = _lib()
    A = S.cases()["random_5000"]
    f = oracle.snap_file_bytes(A, 1)
    for cut in (10, 30, len(f) // 2):
        p = tmp_path / ("t%d.snap" % cut)
        p.write_bytes(f[:cut])
        with pytest.raises(engine.GBError) as ei:
            engine.snap_file_info(str(p))
        assert ei.value.code == engine.GB_ERR_CORRUPT
    with pytest.raises(engine.GBError):
        engine.snap_file_info(str(tmp_path / "missing.snap"))


def test_max_bytes_bounds_the_streams(oracle):
    import ctypes
    engine = _lib()
    for name, A in S.cases().items():
        cap = ctypes.c_int64()
        assert engine.lib().gb_snap_max_bytes(len(A), ctypes.byref(cap)) == 0
        for method in (0, 1):
            total = sum(c[2] for c in oracle.stream_encode(A, method))
            assert total <= cap.value, (name, method, total, cap.value)
