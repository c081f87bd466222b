"""CPU tests of the C-ABI library: it builds for sm_103a, loads, and exports
every function declared in include/gbool.h (no compute without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "gbool.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "defined")))


def test_library_exports_every_declared_symbol():
    from vlsi_layout_gb300 import build as B
    lib = B.build()
    L = ctypes.CDLL(lib)
    names = _declared()
    assert "PerformBoostPolygonOperation" in names and "gb_op_bool" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_engine_refuses_without_library(tmp_path, monkeypatch):
    from vlsi_layout_gb300 import engine
    monkeypatch.setattr(engine, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(engine, "_lib", None)
    try:
        engine.lib()
    except RuntimeError as e:
        assert "no CPU fallback" in str(e)
    else:
        raise AssertionError("engine loaded without its library")


def test_bench_reads_committed_profile_traffic():
    # the bench line's roofline.traffic comes from the committed ncu summary of
    # the scanline kernel; a summary without a parsable figure would drop it
    import sys
    sys.path.insert(0, ROOT)
    import bench
    t = bench.ncu_traffic()
    assert t is not None and t > 1e8
    peak, kind = bench.peaks()
    assert peak > 1000 and kind in ("measured", "fallback")
