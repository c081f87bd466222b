"""CPU tests of the SNAP codec oracle (box codec of box_codec.f90 + Snappy raw
format + .snap file of serialization.f90): the hand-derived known answer,
the golden fixtures (Snappy bytes from the Snappy library), round trips over
the seeded cases, the file layout, and the decoder's desync checks."""
import hashlib
import struct

import numpy as np
import pytest

import snapcases as S


def test_codec_known_answer(oracle):
    g = S.golden()["codec_known_answer"]
    b = np.array(g["boxes"], np.int32)
    raw = oracle.codec_encode_chunk(b)
    assert raw.hex() == g["bytes_hex"]
    assert np.array_equal(oracle.codec_decode_chunk(raw, len(b)), b)


def test_golden_fixtures_decode(oracle):
    for rec in S.golden_layers():
        name, boxes, chunks = rec[:3]
        if len(rec) > 3:
            assert S.sha(boxes_sorted(oracle, boxes)) == rec[3], name
            boxes = boxes_sorted(oracle, boxes)
        parts = []
        for nb, rn, rsha, lib in chunks:
            raw = oracle.snappy_decompress(lib)
            assert len(raw) == rn
            assert hashlib.sha256(raw).hexdigest() == rsha, name
            parts.append(oracle.codec_decode_chunk(raw, nb))
        got = np.concatenate(parts) if parts else np.zeros((0, 4), np.int32)
        assert np.array_equal(got, boxes.reshape(-1, 4)), name


def boxes_sorted(oracle, B):
    return B[np.argsort(oracle.morton_keys_np(B), kind="stable")]


@pytest.mark.parametrize("method", [0, 1])
def test_round_trip(oracle, method):
    for name, A in S.cases().items():
        ch = oracle.stream_encode(A, method)
        assert len(ch) == (len(A) + 65535) // 65536
        assert np.array_equal(oracle.stream_decode(ch, method), A), name


def test_snappy_library_reads_oracle_streams(oracle):
    pa = pytest.importorskip("pyarrow")
    for name, A in S.cases().items():
        for nb, rn, cn, data in oracle.stream_encode(A, 1):
            raw = pa.decompress(data, decompressed_size=rn, codec="snappy", asbytes=True)
            assert len(raw) == rn, name


def test_snappy_decoder_rejects_bad_streams(oracle):
    raw = oracle.codec_encode_chunk(S.cases()["random_5000"])
    data = bytearray(oracle.snappy_compress(raw))
    with pytest.raises(ValueError):
        oracle.snappy_decompress(bytes(data[:len(data) // 2]))  # truncated
    bad = bytearray([5, 0x02 | (3 << 2), 9, 0])  # 5 bytes wanted, a copy from offset 9 of nothing
    with pytest.raises(ValueError):
        oracle.snappy_decompress(bytes(bad))


def test_codec_desync_is_an_error(oracle):
    b = np.array([[0, 0, 10, 10], [0, 0, 12, 10]], np.int32)
    raw = bytearray(oracle.codec_encode_chunk(b))
    # 13 0a | 0f 0c 0a: the second record's new width 12 (varint 0c) becomes
    # index 5 of a one-entry dictionary
    assert bytes(raw).hex() == "130a0f0c0a"
    raw2 = bytes(raw[:2]) + bytes([raw[2] & ~2]) + bytes([5, 0]) + bytes(raw[4:])
    with pytest.raises(ValueError):
        oracle.codec_decode_chunk(raw2, 2)
    with pytest.raises(ValueError):
        oracle.codec_decode_chunk(bytes(raw[:2]), 2)  # stream ends inside the second record


def test_int16_index_wrap_is_not_decodable(oracle):
    # more than 32767 distinct widths: box_codec.f90 writes int(idx, int16), which
    # wraps, and DecompressBoxesUsingCodec stops on the out-of-range index
    A = S.wrap_case()
    raw = oracle.codec_encode_chunk(A)
    with pytest.raises(ValueError):
        oracle.codec_decode_chunk(raw, len(A))


def test_snap_file_layout(oracle):
    A = S.cases()["chunk_plus_one"]
    pn = np.arange(len(A), dtype=np.int64) * 3
    f = oracle.snap_file_bytes(A, 1, layer_properties=1 | 4, pnum=pn)
    ver, props, total, nch, method = struct.unpack_from("<iiqqi", f, 0)
    assert (ver, props, total, nch, method) == (1, 5, len(A), 2, 1)
    # serialization.f90:133-180: the last 8 bytes hold the 1-based position of
    # the offset table, which holds the 1-based positions of the chunk headers
    table = struct.unpack_from("<q", f, len(f) - 8)[0]
    offs = np.frombuffer(f, np.int64, nch, table - 1)
    assert (len(f) - 8 - (table - 1)) == 8 * nch
    assert offs[0] - 1 == 28 + 8 * len(A)
    for o in offs:
        nb, rn, cn = struct.unpack_from("<qqq", f, o - 1)
        assert nb in (65536, 1) and cn > 0
    props2, m2, chunks, pn2 = oracle.snap_file_parse(f)
    assert props2 == 5 and m2 == 1 and np.array_equal(pn2, pn)
    assert np.array_equal(oracle.stream_decode(chunks, m2), A)
