"""ctypes wrapper of the CPU oracle (gbo_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py, always as the checker or the timed
CPU baseline.  The product package never imports this module.

Boxes are numpy int32 arrays of shape (n, 4) holding x1, y1, x2, y2.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "_build", "libgbo_oracle.so")
_REF = os.path.join(_HERE, "_ref", "libref_sort.so")

XOR, OR, AND, NOT, MERGE = 0, 1, 2, 3, 4
OVERLAP = 7  # single-layer AND: area covered by at least two boxes

_lib = None


def build(force=False):
    """Compile the oracle (and the reference CPU sort helpers when mounted)."""
    subprocess.check_call(["make", "-s", "-C", _HERE, "_build/libgbo_oracle.so"] + (["-B"] if force else []))
    subprocess.call(["make", "-s", "-C", _HERE, "ref"], stdout=subprocess.DEVNULL)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB):
            build()
        L = ctypes.CDLL(_LIB)
        P = ctypes.c_void_p
        i64, i32 = ctypes.c_int64, ctypes.c_int32
        L.orc_boolean.argtypes = [P, i64, P, i64, ctypes.c_int, ctypes.c_int, ctypes.POINTER(P)]
        L.orc_boolean.restype = i64
        L.orc_grow.argtypes = [P, i64, i32, i32, i32, i32, ctypes.c_int, ctypes.POINTER(P)]
        L.orc_grow.restype = i64
        L.orc_size.argtypes = [P, i64, i32, ctypes.c_int, ctypes.POINTER(P)]
        L.orc_size.restype = i64
        L.orc_union_area.argtypes = [P, i64]
        L.orc_union_area.restype = i64
        L.orc_components.argtypes = [P, i64, P]
        L.orc_components.restype = i64
        L.orc_interactions.argtypes = [P, i64, P, P, P]
        L.orc_interactions.restype = None
        L.orc_component_areas.argtypes = [P, i64, P]
        L.orc_component_areas.restype = i64
        L.orc_morton_key.argtypes = [P]
        L.orc_morton_key.restype = ctypes.c_uint64
        L.orc_tracker_key.argtypes = [i32, i32]
        L.orc_tracker_key.restype = ctypes.c_uint64
        L.orc_um_to_dbu.argtypes = [ctypes.c_double]
        L.orc_um_to_dbu.restype = i32
        L.orc_op1.argtypes = [P, i64, i32, ctypes.c_int, P, P]
        L.orc_op1.restype = None
        L.orc_op1_cells.argtypes = [P, P, i64, i32, ctypes.c_int, P, P]
        L.orc_op1_cells.restype = None
        L.orc_codec_encode.argtypes = [P, i64, P]
        L.orc_codec_encode.restype = i64
        L.orc_codec_decode.argtypes = [P, i64, i64, P]
        L.orc_codec_decode.restype = i64
        L.orc_snappy_max_length.argtypes = [i64]
        L.orc_snappy_max_length.restype = i64
        L.orc_snappy_compress.argtypes = [P, i64, P]
        L.orc_snappy_compress.restype = i64
        L.orc_snappy_uncompressed_length.argtypes = [P, i64]
        L.orc_snappy_uncompressed_length.restype = i64
        L.orc_snappy_decompress.argtypes = [P, i64, P, i64]
        L.orc_snappy_decompress.restype = i64
        L.orc_op1_digest.argtypes = [P, i64, i32, ctypes.c_int, P, P, P]
        L.orc_op1_digest.restype = None
        L.orc_op1_cells_digest.argtypes = [P, P, i64, i32, ctypes.c_int, P, P, P]
        L.orc_op1_cells_digest.restype = None
        L.orc_strip_hash.argtypes = [i32, i32, i32, i32]
        L.orc_strip_hash.restype = ctypes.c_uint64
        L.orc_strip_digest.argtypes = [P, i64]
        L.orc_strip_digest.restype = ctypes.c_uint64
        L.orc_refpath_op1_cells.argtypes = [P, P, i64, i32, P, P]
        L.orc_refpath_op1_cells.restype = None
        L.orc_refpath_op1_layer.argtypes = [P, i64, i32, ctypes.c_int, ctypes.POINTER(P)]
        L.orc_refpath_op1_layer.restype = i64
        L.orc_refpath_subtract.argtypes = [P, P, P]
        L.orc_refpath_subtract.restype = i64
        L.orc_free.argtypes = [P]
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _arr(b):
    b = np.ascontiguousarray(b, dtype=np.int32).reshape(-1, 4)
    return b


def _take(n, p):
    if n < 0:
        raise ValueError("oracle rejected an invalid box")
    if n == 0:
        lib().orc_free(p)
        return np.zeros((0, 4), np.int32)
    out = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_int32)), shape=(n * 4,))
    res = out.copy().reshape(n, 4)
    lib().orc_free(p)
    return res


def boolean(A, B, op, grid_log2=16):
    A, B = _arr(A), _arr(B)
    p = ctypes.c_void_p()
    n = lib().orc_boolean(A.ctypes.data, len(A), B.ctypes.data, len(B), op, grid_log2, ctypes.byref(p))
    return _take(n, p)


def merge(A, grid_log2=16):
    return boolean(A, np.zeros((0, 4), np.int32), MERGE, grid_log2)


def grow(A, E, N, W, S, grid_log2=16):
    A = _arr(A)
    p = ctypes.c_void_p()
    n = lib().orc_grow(A.ctypes.data, len(A), E, N, W, S, grid_log2, ctypes.byref(p))
    return _take(n, p)


def size(A, s, grid_log2=16):
    A = _arr(A)
    p = ctypes.c_void_p()
    n = lib().orc_size(A.ctypes.data, len(A), s, grid_log2, ctypes.byref(p))
    return _take(n, p)


def union_area(A):
    A = _arr(A)
    return int(lib().orc_union_area(A.ctypes.data, len(A)))


def components(A):
    A = _arr(A)
    labels = np.zeros(len(A), np.int64)
    n = lib().orc_components(A.ctypes.data, len(A), labels.ctypes.data)
    return int(n), labels


def overlap(A, grid_log2=16):
    """Single-layer AND (design_impl.f90:385-498) as canonical strips of the
    area covered by at least two boxes of A."""
    return boolean(A, np.zeros((0, 4), np.int32), OVERLAP, grid_log2)


def interactions(A):
    """(strict overlap pairs, singletons, singleton mask) of one layer."""
    A = _arr(A)
    pairs, singles = ctypes.c_int64(), ctypes.c_int64()
    mask = np.zeros(len(A), np.uint8)
    lib().orc_interactions(A.ctypes.data, len(A), ctypes.byref(pairs), ctypes.byref(singles), mask.ctypes.data)
    return int(pairs.value), int(singles.value), mask


def component_areas(A):
    """Union area per PNUM component: [singleton area, area of component 1, ...]."""
    A = _arr(A)
    R = int(lib().orc_component_areas(A.ctypes.data, len(A), None))
    out = np.zeros(R + 1, np.int64)
    lib().orc_component_areas(A.ctypes.data, len(A), out.ctypes.data)
    return out


def morton_keys(A):
    A = _arr(A)
    L = lib()
    return np.array([L.orc_morton_key(A[i:i + 1].ctypes.data) for i in range(len(A))], np.uint64)


def morton_keys_np(A):
    """Vectorised restatement of the same key (numpy), for large arrays."""
    A = _arr(A).astype(np.int64)
    cx = ((A[:, 0] + A[:, 2]) // 2)
    cy = ((A[:, 1] + A[:, 3]) // 2)
    # C division truncates toward zero; numpy // floors: fix negative odd sums.
    sx = A[:, 0] + A[:, 2]
    sy = A[:, 1] + A[:, 3]
    cx = np.where((sx < 0) & (sx % 2 != 0), cx + 1, cx)
    cy = np.where((sy < 0) & (sy % 2 != 0), cy + 1, cy)
    ux = (cx.astype(np.uint64) & np.uint64(0xFFFFFFFF)) ^ np.uint64(0x80000000)
    uy = (cy.astype(np.uint64) & np.uint64(0xFFFFFFFF)) ^ np.uint64(0x80000000)

    def spread(m):
        m = (m | (m << np.uint64(16))) & np.uint64(0x0000FFFF0000FFFF)
        m = (m | (m << np.uint64(8))) & np.uint64(0x00FF00FF00FF00FF)
        m = (m | (m << np.uint64(4))) & np.uint64(0x0F0F0F0F0F0F0F0F)
        m = (m | (m << np.uint64(2))) & np.uint64(0x3333333333333333)
        m = (m | (m << np.uint64(1))) & np.uint64(0x5555555555555555)
        return m

    return (spread(uy) << np.uint64(1)) | spread(ux)


def tracker_keys_np(X, Y):
    ux = (np.asarray(X, np.int64).astype(np.uint64) & np.uint64(0xFFFFFFFF)) ^ np.uint64(0x80000000)
    uy = (np.asarray(Y, np.int64).astype(np.uint64) & np.uint64(0xFFFFFFFF)) ^ np.uint64(0x80000000)
    return (ux << np.uint64(32)) | uy


def um_to_dbu(r):
    return int(lib().orc_um_to_dbu(float(r)))


def op1(A, amount=1, grid_log2=16):
    """OP1 deck; returns (counts dict, union area)."""
    A = _arr(A)
    counts = np.zeros(8, np.int64)
    area = np.zeros(1, np.int64)
    lib().orc_op1(A.ctypes.data, len(A), amount, grid_log2, counts.ctypes.data, area.ctypes.data)
    keys = ["poly_1", "poly_2", "outer_ring", "inner_ring", "ring_and1", "ring_intersection", "merged"]
    return {k: int(counts[i]) for i, k in enumerate(keys)}, int(area[0])


def op1_cells(A, off, amount=1, grid_log2=16):
    """OP1 on every cell (cells in parallel on all OpenMP threads).
    Returns counts[ncell, 6] (poly_1, poly_2, outer, inner, and1, inter) and
    the union area per cell."""
    A = _arr(A)
    off = np.ascontiguousarray(off, np.int64)
    ncell = len(off) - 1
    counts = np.zeros((ncell, 8), np.int64)
    area = np.zeros(ncell, np.int64)
    lib().orc_op1_cells(A.ctypes.data, off.ctypes.data, ncell, amount, grid_log2, counts.ctypes.data,
                        area.ctypes.data)
    return counts[:, :6], area


def op1_digest(A, amount=1, grid_log2=16):
    """OP1 on one layer (each operator parallel over its tiles): returns
    (counts[6], area, digests[7]) with digests of poly_1, poly_2, outer,
    inner, and1, inter and merged(P)."""
    A = _arr(A)
    counts = np.zeros(8, np.int64)
    area = np.zeros(1, np.int64)
    dig = np.zeros(7, np.uint64)
    lib().orc_op1_digest(A.ctypes.data, len(A), amount, grid_log2, counts.ctypes.data, area.ctypes.data,
                         dig.ctypes.data)
    return counts[:6], int(area[0]), dig


def op1_cells_digest(A, off, amount=1, grid_log2=16):
    """op1_cells plus per-cell strip digests: returns counts[ncell, 6],
    area[ncell] and digests[ncell, 7] (uint64: poly_1, poly_2, outer, inner,
    and1, inter, merged(P))."""
    A = _arr(A)
    off = np.ascontiguousarray(off, np.int64)
    ncell = len(off) - 1
    counts = np.zeros((ncell, 8), np.int64)
    area = np.zeros(ncell, np.int64)
    dig = np.zeros((ncell, 7), np.uint64)
    lib().orc_op1_cells_digest(A.ctypes.data, off.ctypes.data, ncell, amount, grid_log2, counts.ctypes.data,
                               area.ctypes.data, dig.ctypes.data)
    return counts[:, :6], area, dig


def strip_digest(A):
    """Order-independent digest of a strip list (sum mod 2^64 of strip_hash)."""
    A = _arr(A)
    return int(lib().orc_strip_digest(A.ctypes.data, len(A)))


def strip_digests_by_cell(A, off):
    """strip_digest of every cell's slice A[off[k]:off[k+1]] (uint64 array)."""
    A = _arr(A)
    return np.array([strip_digest(A[off[k]:off[k + 1]]) for k in range(len(off) - 1)], np.uint64)


def refpath_op1_cells(A, off, amount=1):
    """The reference's CPU path for OP1 (gbo_refpath.cpp) on every cell, cells
    in parallel: counts[ncell, 6] in the reference's decompositions and the
    union area per cell."""
    A = _arr(A)
    off = np.ascontiguousarray(off, np.int64)
    ncell = len(off) - 1
    counts = np.zeros((ncell, 6), np.int64)
    area = np.zeros(ncell, np.int64)
    lib().orc_refpath_op1_cells(A.ctypes.data, off.ctypes.data, ncell, amount, counts.ctypes.data, area.ctypes.data)
    return counts, area


def refpath_op1_layer(A, which, amount=1):
    """Layer `which` (0 poly_1, 1 poly_2, 2 outer, 3 inner, 4 and1, 5 inter) of
    the reference's CPU path for OP1, as the reference decomposes it."""
    A = _arr(A)
    p = ctypes.c_void_p()
    n = lib().orc_refpath_op1_layer(A.ctypes.data, len(A), amount, which, ctypes.byref(p))
    return _take(n, p)


def refpath_subtract(subject, clip):
    """SubtractBox: subject minus clip as up to four boxes."""
    s, c = _arr([subject]), _arr([clip])
    out = np.zeros((4, 4), np.int32)
    k = lib().orc_refpath_subtract(s.ctypes.data, c.ctypes.data, out.ctypes.data)
    return out[:k]


def canonical(A):
    """Sort boxes by (x1, y1, x2, y2)."""
    A = _arr(A)
    if len(A) == 0:
        return A
    idx = np.lexsort((A[:, 3], A[:, 2], A[:, 1], A[:, 0]))
    return A[idx]


def area_of(A):
    A = _arr(A).astype(np.int64)
    return int(((A[:, 2] - A[:, 0]) * (A[:, 3] - A[:, 1])).sum())


def xor_empty(A, B, grid_log2=16):
    """Our XOR checker (stands in for boost_xor_checker.cpp:68-152): True iff
    the point sets of A and B are equal."""
    return len(boolean(A, B, XOR, grid_log2)) == 0


def ref_sort_lib():
    """The reference's own CPU sort helpers (gpu_morton.cu / event_sorter.cu,
    #ifndef USE_GPU branch), compiled from the mounted sources into _ref/ by
    the Makefile.  None when they were not built."""
    if not os.path.exists(_REF):
        return None
    L = ctypes.CDLL(_REF)
    L.thrust_sort_boxes_direct.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    L.thrust_sort_boxes_indirect.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    L.cpp_std_sort_trackers.argtypes = [ctypes.c_void_p, ctypes.c_int64]
    return L


# ---------------------------------------------------------------- SNAP codec
# box_codec.f90 (BoxCodecModule) and serialization.f90; see gbo_snap.cpp.
BOXES_PER_CHUNK = 65536          # box_codec.f90:227
CODEC_VERSION = 1                # commonmodule.f90:22
METHOD_NONE, METHOD_SNAPPY = 0, 1  # box_codec.f90:228-233
LAYER_STATE_PNUM = 4             # design.f90:41


def _u8(b):
    return np.frombuffer(bytes(b), np.uint8) if not isinstance(b, np.ndarray) else np.ascontiguousarray(b, np.uint8)


def codec_encode_chunk(A):
    """CompressBoxesUsingCodec on one chunk: the raw codec bytes."""
    A = _arr(A)
    out = np.zeros(32 * len(A) + 1, np.uint8)
    k = lib().orc_codec_encode(A.ctypes.data, len(A), out.ctypes.data)
    return out[:k].tobytes()


def codec_decode_chunk(raw, n):
    """DecompressBoxesUsingCodec: n boxes from raw codec bytes (ValueError on desync)."""
    r = _u8(raw)
    out = np.zeros((n, 4), np.int32)
    k = lib().orc_codec_decode(r.ctypes.data, len(r), n, out.ctypes.data)
    if k != 0:
        raise ValueError("codec stream desync at record %d" % (-k - 1))
    return out


def snappy_compress(raw):
    r = _u8(raw)
    out = np.zeros(lib().orc_snappy_max_length(len(r)), np.uint8)
    k = lib().orc_snappy_compress(r.ctypes.data, len(r), out.ctypes.data)
    return out[:k].tobytes()


def snappy_decompress(data):
    d = _u8(data)
    n = lib().orc_snappy_uncompressed_length(d.ctypes.data, len(d))
    if n < 0:
        raise ValueError("bad snappy preamble")
    out = np.zeros(max(n, 1), np.uint8)
    k = lib().orc_snappy_decompress(d.ctypes.data, len(d), out.ctypes.data, n)
    if k != n:
        raise ValueError("malformed snappy stream")
    return out[:n].tobytes()


def stream_encode(A, method=METHOD_SNAPPY):
    """CompressBoxesToStream (box_codec.f90:675-760): per chunk
    (num_boxes, raw_byte_size, compressed_size, data)."""
    A = _arr(A)
    chunks = []
    for c0 in range(0, len(A), BOXES_PER_CHUNK):
        part = A[c0:c0 + BOXES_PER_CHUNK]
        raw = codec_encode_chunk(part)
        data = snappy_compress(raw) if method == METHOD_SNAPPY else raw
        chunks.append((len(part), len(raw), len(data), data))
    return chunks


def stream_decode(chunks, method=METHOD_SNAPPY):
    """DecompressStreamToBoxes (box_codec.f90:765-880)."""
    parts = []
    for nb, raw_n, comp_n, data in chunks:
        raw = snappy_decompress(data) if method == METHOD_SNAPPY else bytes(data)
        if len(raw) != raw_n:
            raise ValueError("raw size differs from the chunk header")
        parts.append(codec_decode_chunk(raw, nb))
    return np.concatenate(parts) if parts else np.zeros((0, 4), np.int32)


def snap_file_bytes(A, method=METHOD_SNAPPY, layer_properties=0, pnum=None):
    """SaveCompressedStreamToDisk (serialization.f90:15-50): int32 version,
    int32 layer properties, int64 total boxes, int64 chunks, int32 method,
    [int64 PNUM table], then per chunk three int64 and the data, then the
    int64 table of the chunks' 1-based file positions and, last, the int64
    1-based position of that table."""
    import struct
    chunks = stream_encode(A, method)
    out = bytearray(struct.pack("<iiqqi", CODEC_VERSION, layer_properties, len(_arr(A)), len(chunks), method))
    if pnum is not None:
        out += np.ascontiguousarray(pnum, np.int64).tobytes()
    offs = []
    for nb, raw_n, comp_n, data in chunks:
        offs.append(len(out) + 1)
        out += struct.pack("<qqq", nb, raw_n, comp_n) + bytes(data)
    table = len(out) + 1
    out += np.array(offs, np.int64).tobytes() + struct.pack("<q", table)
    return bytes(out)


def snap_file_parse(buf):
    """RestoreCompressedStreamFromDisk (serialization.f90:56-130):
    (layer_properties, method, chunks, pnum or None)."""
    import struct
    ver, props, total, nch, method = struct.unpack_from("<iiqqi", buf, 0)
    p = 28
    pnum = None
    if props & LAYER_STATE_PNUM:
        pnum = np.frombuffer(buf, np.int64, total, p).copy()
        p += 8 * total
    chunks = []
    for _ in range(nch):
        nb, raw_n, comp_n = struct.unpack_from("<qqq", buf, p)
        p += 24
        chunks.append((nb, raw_n, comp_n, bytes(buf[p:p + comp_n])))
        p += comp_n
    return props, method, chunks, pnum
