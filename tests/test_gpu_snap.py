"""GPU parity of the SNAP layer streams (gb_compress_boxes_to_stream,
gb_decompress_stream_to_boxes, gb_save_layer_to_snap,
gb_restore_snap_to_layer) against the oracle: codec bytes and Snappy bytes
bit-exact per chunk, decoding of the oracle's and the Snappy library's
streams, .snap files byte-identical, and malformed input reported as
GB_ERR_CORRUPT with the context still usable."""
import os

import numpy as np
import pytest

import snapcases as S

pytestmark = pytest.mark.gpu


def _sorted(oracle, B):
    return B[np.argsort(oracle.morton_keys_np(B), kind="stable")]


def test_codec_known_answer(ctx):
    g = S.golden()["codec_known_answer"]
    b = np.array(g["boxes"], np.int32)
    ch = ctx.compress_boxes_to_stream(b, method=0)
    assert len(ch) == 1 and ch[0][3].hex() == g["bytes_hex"]
    assert np.array_equal(ctx.decompress_stream_to_boxes(ch, 0), b)


@pytest.mark.parametrize("method", [0, 1])
def test_stream_parity(ctx, oracle, method):
    for name, A in S.cases(big=True).items():
        got = ctx.compress_boxes_to_stream(A, method)
        exp = oracle.stream_encode(A, method)
        assert len(got) == len(exp), name
        for k, (g, e) in enumerate(zip(got, exp)):
            assert g[:3] == e[:3], (name, k, g[:3], e[:3])
            assert g[3] == e[3], (name, k)
        assert np.array_equal(ctx.decompress_stream_to_boxes(got, method), A), name


def test_decodes_oracle_and_library_streams(ctx, oracle):
    for rec in S.golden_layers():
        name, boxes, chunks = rec[:3]
        if len(rec) > 3:
            boxes = _sorted(oracle, boxes)
            assert S.sha(boxes) == rec[3], name
        boxes = boxes.reshape(-1, 4)
        lib_chunks = [(nb, rn, len(data), data) for nb, rn, _, data in chunks]
        got = ctx.decompress_stream_to_boxes(lib_chunks, 1)
        assert np.array_equal(got, boxes), name
        assert np.array_equal(ctx.decompress_stream_to_boxes(oracle.stream_encode(boxes, 1), 1), boxes), name


def test_wrapped_index_matches_the_reference_format(ctx, oracle):
    # more than 32767 distinct widths in a chunk: the bytes still match the
    # reference's encoding (wrapped int16 index), and both decoders refuse them
    from vlsi_layout_gb300 import engine
    A = S.wrap_case()
    got = ctx.compress_boxes_to_stream(A, 0)
    assert got[0][3] == oracle.codec_encode_chunk(A)
    with pytest.raises(engine.GBError) as ei:
        ctx.decompress_stream_to_boxes(got, 0)
    assert ei.value.code == engine.GB_ERR_CORRUPT
    with pytest.raises(ValueError):
        oracle.codec_decode_chunk(got[0][3], len(A))
    ctx.sync()


def test_snap_file(ctx, oracle, tmp_path):
    from vlsi_layout_gb300 import engine
    A = S.cases()["chunk_plus_one"]
    pn = np.arange(len(A), dtype=np.int64) * 7 - 3
    for method, props, pnum in ((1, 1 | 2, pn), (0, 0, None), (1, 8 | 32, None)):
        p = str(tmp_path / ("l%d_%d.snap" % (method, props)))
        ctx.save_layer_to_snap(p, A, method, props, pnum)
        want_props = (props & ~8 & ~4) | (4 if pnum is not None else 0)
        exp = oracle.snap_file_bytes(A, method, want_props, pnum)
        assert open(p, "rb").read() == exp
        assert engine.snap_file_info(p) == (len(A), 2, method, want_props)
        b, props2, m2, pn2 = ctx.restore_snap_to_layer(p)
        assert np.array_equal(b, A) and props2 == want_props and m2 == method
        assert (pn2 is None) == (pnum is None)
        if pnum is not None:
            assert np.array_equal(pn2, pnum)
    # a file written by the oracle; an empty file is an empty layer
    q = str(tmp_path / "oracle.snap")
    B = S.cases()["stdcell"]
    with open(q, "wb") as fh:
        fh.write(oracle.snap_file_bytes(B, 1))
    assert np.array_equal(ctx.restore_snap_to_layer(q)[0], B)
    e = str(tmp_path / "empty.snap")
    open(e, "wb").close()
    assert len(ctx.restore_snap_to_layer(e)[0]) == 0
    z = str(tmp_path / "zero.snap")
    ctx.save_layer_to_snap(z, np.zeros((0, 4), np.int32))
    assert open(z, "rb").read() == oracle.snap_file_bytes(np.zeros((0, 4), np.int32), 1)


def test_malformed_streams_are_errors(ctx, oracle):
    from vlsi_layout_gb300 import engine
    A = S.cases()["random_5000"]
    nb, rn, cn, data = oracle.stream_encode(A, 1)[0]
    bad = [
        [(nb, rn, cn // 2, data[:cn // 2])],                       # truncated Snappy stream
        [(nb, rn + 1, cn, data)],                                  # header disagrees with the preamble
        [(nb, rn, 4, bytes([rn & 127 | 128, rn >> 7 & 127 | 128, rn >> 14, 0x02 | 3 << 2]))],  # copy past input
    ]
    raw = oracle.codec_encode_chunk(A)
    bad0 = [[(nb, rn // 2, rn // 2, raw[:rn // 2])],                # codec stream ends early
            [(nb + 5, rn, rn, raw)]]                                # more boxes than records
    for chunks, m in [(c, 1) for c in bad] + [(c, 0) for c in bad0]:
        with pytest.raises(engine.GBError) as ei:
            ctx.decompress_stream_to_boxes(chunks, m)
        assert ei.value.code == engine.GB_ERR_CORRUPT, chunks[0][:3]
    # the context is still usable
    assert np.array_equal(ctx.decompress_stream_to_boxes(oracle.stream_encode(A, 1), 1), A)
    with pytest.raises(engine.GBError):
        ctx.compress_boxes_to_stream(A, 2)  # ZLIB is not supported
