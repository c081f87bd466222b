"""Control decks run through gb_run_deck (the MAGPARSER interpreter on the GPU
engine): the README's OP1 ring check via RUN_LOOP, flushed outputs checked
against the oracle, ASSERT_ZERO failures counted, bad decks refused; layer
files read and written as the reference does (KLBIN and SNAP sections,
RestoreSnapToLayer's ".bin" rule, invalid boxes refused, missing files as
empty layers with temporary_layers 2, memory layers flushed to SNAP files and
read back, output layers written to the files their .mag names)."""
import os

import numpy as np
import pytest

from gen import random_layer

pytestmark = pytest.mark.gpu

DECK = """# Control file for MAGPARSER
include(`./src/op_template.m4')dnl
program ringcheck
systeminfo
var temp_folder mkTempFolder
var abort_on_assert_zero 1
var temporary_layers 2
decl design d1 = design.mag
decl output o1 = out.mag
decl memory t1 = nothing
info
exec init t1:nothing
RUN_LOOP(`OP1',`t1',`d1',`poly',`0.001',`li1',`0.001',`met1',`0.001',`met2',`0.001')dnl
exec run o1:ring = t1:poly_outer_ring + d1:li1
exec run o1:x = d1:met1 ^ d1:met2
exec run o1:ext = d1:poly EXTENT t1:nothing
exec run o1:g = d1:met1 GROW t1:nothing 0.002 0.0 0.0035 0.001
exec run o1:s = d1:li1 SIZE t1:nothing -0.002
exec run o1:a = d1:met1 * d1:met2
exec run o1:n = d1:met1 @ d1:met2
flush
end
"""


def _write_mag(path, layers, klbin=()):
    with open(path, "w") as fh:
        fh.write("magic\ntech sky130A\n")
        for name, b in layers.items():
            fh.write("<< %s >>\n" % name)
            if name in klbin:
                side = name + ".bin"
                b.astype("<i4").tofile(os.path.join(os.path.dirname(path), side))
                fh.write("KLBIN %s\n" % side)
            else:
                for r in b:
                    fh.write("rect %d %d %d %d\n" % tuple(r))
        fh.write("<< labels >>\nrlabel metal1 0 0 1 1 0 A\n<< end >>\n")


def _read_mag(path):
    out, sec = {}, None
    base = os.path.dirname(path)
    for line in open(path):
        line = line.strip()
        if line.startswith("<< end"):
            break
        if line.startswith("<<"):
            sec = line[2:].split(">>")[0].strip()
            out[sec] = []
        elif line.startswith("rect") and sec:
            out[sec].append([int(v) for v in line.split()[1:5]])
        elif line.startswith("KLBIN") and sec:
            p = line.split()[1]
            p = p if os.path.isabs(p) else os.path.join(base, p)
            out[sec] = np.fromfile(p, "<i4").reshape(-1, 4).tolist()
    return {k: np.array(v, np.int32).reshape(-1, 4) for k, v in out.items()}


def _canon(b):
    return b[np.lexsort((b[:, 3], b[:, 2], b[:, 1], b[:, 0]))] if len(b) else b


def _read_snap(oracle, path):
    props, method, chunks, _ = oracle.snap_file_parse(open(path, "rb").read())
    return oracle.stream_decode(chunks, method).reshape(-1, 4) if chunks else np.zeros((0, 4), np.int32)


def test_readme_ring_deck(tmp_path, monkeypatch, oracle):
    from vlsi_layout_gb300 import engine
    monkeypatch.chdir(tmp_path)
    L = {"poly": random_layer(4000, die=300000, seed=41), "li1": random_layer(4000, die=300000, seed=42),
         "met1": random_layer(4000, die=300000, seed=43), "met2": random_layer(4000, die=300000, seed=44)}
    _write_mag(str(tmp_path / "design.mag"), L, klbin=("met2",))
    (tmp_path / "deck.ctr").write_text(DECK)
    rc, log, fails = engine.run_deck(str(tmp_path / "deck.ctr"))
    assert rc == 0, log
    assert fails == 0, log
    assert log.count("ASSERT_ZERO") == 8 and "fail" not in log
    out = _read_mag(str(tmp_path / "out.mag"))
    O = oracle
    outer = O.boolean(O.grow(L["poly"], 1, 1, 1, 1), L["poly"], O.NOT)
    assert np.array_equal(_canon(out["ring"]), O.boolean(outer, L["li1"], O.OR))
    assert np.array_equal(_canon(out["x"]), O.boolean(L["met1"], L["met2"], O.XOR))
    p = L["poly"]
    assert out["ext"].tolist() == [[p[:, 0].min(), p[:, 1].min(), p[:, 2].max(), p[:, 3].max()]]
    # GROW east 0.002, north 0.0, west 0.0035 -> int(3.5) = 3, south 0.001 (controlparser.f90:568-570)
    assert np.array_equal(_canon(out["g"]), O.grow(L["met1"], 2, 0, 3, 1))
    assert np.array_equal(_canon(out["s"]), O.size(L["li1"], -2))
    assert np.array_equal(_canon(out["a"]), O.boolean(L["met1"], L["met2"], O.AND))
    assert np.array_equal(_canon(out["n"]), O.boolean(L["met1"], L["met2"], O.NOT))
    # temporary_layers 2: memory layers are flushed to SNAP files named temp_folder + design + "_MTL_" + layer
    spilled = _read_snap(O, str(tmp_path / "mkTempFoldert1_MTL_poly_outer_ring"))
    assert np.array_equal(_canon(spilled), outer)
    assert not (tmp_path / "mkTempFoldert1_MTL_poly_ring_and1").exists()  # empty layers are not written


SNAP_DECK = """program ingest
var temporary_layers 2
var temp_folder tmp_
decl design d1 = design.mag
decl output o1 = out.mag
decl memory t1 = nothing
exec init t1:nothing
exec run t1:u = d1:poly + d1:li1
exec run t1:n = d1:met1 ~ d1:poly
exec run t1:e = d1:gone + d1:li1
flush
exec run o1:ring = t1:u ^ d1:met1
exec run o1:x = t1:n * d1:li1
flush
end
"""


def test_deck_snap_klbin_ingest_and_flush(tmp_path, monkeypatch, oracle):
    """A .mag with a SNAP section, a KLBIN .bin section, rect lines and a missing
    file; memory layers flushed to SNAP and read back by later statements;
    output layers written to the SNAP / KLBin files the output .mag names."""
    from vlsi_layout_gb300 import engine
    O = oracle
    monkeypatch.chdir(tmp_path)
    L = {"poly": random_layer(6000, die=300000, seed=51), "li1": random_layer(6000, die=300000, seed=52),
         "met1": random_layer(3000, die=300000, seed=53)}
    (tmp_path / "poly.snap").write_bytes(O.snap_file_bytes(L["poly"]))
    L["li1"].astype("<i4").tofile(str(tmp_path / "li1.bin"))
    with open(tmp_path / "design.mag", "w") as fh:
        fh.write("magic\n<< poly >>\nSNAP poly.snap\n<< li1 >>\nKLBIN li1.bin\n<< met1 >>\n")
        for r in L["met1"]:
            fh.write("rect %d %d %d %d\n" % tuple(r))
        fh.write("<< gone >>\nKLBIN gone.bin\n<< end >>\n")
    (tmp_path / "out.mag").write_text("magic\n<< ring >>\nSNAP ring.snap\n<< x >>\nKLBIN x.bin\n<< end >>\n")
    (tmp_path / "deck.ctr").write_text(SNAP_DECK)
    rc, log, fails = engine.run_deck(str(tmp_path / "deck.ctr"))
    assert rc == 0, log
    u = O.boolean(L["poly"], L["li1"], O.OR)
    n = O.boolean(L["met1"], L["poly"], O.NOT)
    # memory layers went to SNAP files on the first flush ...
    assert np.array_equal(_canon(_read_snap(O, str(tmp_path / "tmp_t1_MTL_u"))), u)
    assert np.array_equal(_canon(_read_snap(O, str(tmp_path / "tmp_t1_MTL_n"))), n)
    # ... a missing KLBIN file was an empty layer (temporary_layers 2), so e = li1
    assert np.array_equal(_canon(_read_snap(O, str(tmp_path / "tmp_t1_MTL_e"))), O.merge(L["li1"]))
    # ... and were read back for the statements after it; outputs went to their files
    ring = _read_snap(O, str(tmp_path / "ring.snap"))
    assert np.array_equal(_canon(ring), O.boolean(u, L["met1"], O.XOR))
    x = np.fromfile(str(tmp_path / "x.bin"), "<i4").reshape(-1, 4)
    assert np.array_equal(_canon(x), O.boolean(n, L["li1"], O.AND))


def test_deck_file_refusals(tmp_path, monkeypatch):
    """An invalid box in a KLBin file refuses the file (kldata.f90:56); a missing
    file is an error unless temporary_layers 2; an output layer the output .mag
    does not name has no supported file (magparser.f90:548-552)."""
    from vlsi_layout_gb300 import engine
    monkeypatch.chdir(tmp_path)
    np.array([[0, 0, 10, 10], [5, 5, 5, 10]], "<i4").tofile(str(tmp_path / "bad.bin"))
    (tmp_path / "bad.mag").write_text("magic\n<< poly >>\nKLBIN bad.bin\n<< end >>\n")
    (tmp_path / "a.ctr").write_text("program a\ndecl design d1 = bad.mag\nend\n")
    rc, log, _ = engine.run_deck(str(tmp_path / "a.ctr"))
    assert rc == engine.GB_ERR_INVALID_BOX and "INVALID BOX" in log
    (tmp_path / "miss.mag").write_text("magic\n<< poly >>\nKLBIN none.bin\n<< end >>\n")
    (tmp_path / "b.ctr").write_text("program b\ndecl design d1 = miss.mag\nend\n")
    rc, log, _ = engine.run_deck(str(tmp_path / "b.ctr"))
    assert rc == engine.GB_ERR_ARG and "does not exist" in log
    (tmp_path / "c.ctr").write_text("program c\nvar temporary_layers 2\ndecl design d1 = miss.mag\nend\n")
    rc, log, _ = engine.run_deck(str(tmp_path / "c.ctr"))
    assert rc == 0, log
    _write_mag(str(tmp_path / "d.mag"), {"poly": random_layer(300, die=20000, seed=45)})
    (tmp_path / "o.mag").write_text("magic\n<< ring >>\nSNAP ring.snap\n<< end >>\n")
    (tmp_path / "d.ctr").write_text("program d\ndecl design d1 = d.mag\ndecl output o1 = o.mag\n"
                                    "exec run o1:other = d1:poly + d1:poly\nflush\nend\n")
    rc, log, _ = engine.run_deck(str(tmp_path / "d.ctr"))
    assert rc == engine.GB_ERR_ARG and "DBOUT only supports KLBIN" in log


def test_assert_zero_failure_and_errors(tmp_path, monkeypatch):
    from vlsi_layout_gb300 import engine
    monkeypatch.chdir(tmp_path)
    _write_mag(str(tmp_path / "d.mag"), {"poly": random_layer(300, die=20000, seed=45)})
    (tmp_path / "a.ctr").write_text("program a\ndecl design d1 = d.mag\ndecl memory t1 = nothing\n"
                                    "exec init t1:nothing\n"
                                    "exec run t1:nothing = d1:poly ASSERT_ZERO t1:nothing\nend\n")
    rc, log, fails = engine.run_deck(str(tmp_path / "a.ctr"))
    assert rc == 0 and fails == 1 and "ASSERT_ZERO fail" in log
    (tmp_path / "b.ctr").write_text("program b\ndecl design d1 = d.mag\ndecl memory t1 = nothing\n"
                                    "exec init t1:nothing\nexec run t1:x = d1:li1 * d1:poly\nend\n")
    rc, log, fails = engine.run_deck(str(tmp_path / "b.ctr"))
    assert rc == engine.GB_ERR_ARG and "layer not found" in log
    (tmp_path / "c.ctr").write_text("program c\nvar abort_on_xor 1\ndecl design d1 = d.mag\n"
                                    "decl memory t1 = nothing\nexec init t1:nothing\n"
                                    "exec run t1:g = d1:poly GROW t1:nothing 0.001 0.001 0.001 0.001\n"
                                    "exec run t1:x = d1:poly ^ t1:g\nend\n")
    rc, log, fails = engine.run_deck(str(tmp_path / "c.ctr"))
    assert rc == engine.GB_ERR_ARG and "abort_on_xor" in log
