"""Python binding of libgbool.so (ctypes over the C-ABI in include/gbool.h).

This mirrors the reference's operator surface for the box-Boolean path:
layers of int32 boxes and the MAGPARSER operators on them (GROW, SIZE,
AND '*', NOT '~', OR '+', XOR '^', MERGE, ASSERT_ZERO), Klee's-measure area,
PNUM connectivity and the Morton / tracker sorts.  All compute runs in the
CUDA library; if the library is missing this module raises, it never falls
back to a CPU path.

Boxes are numpy int32 arrays of shape (n, 4): x1, y1, x2, y2 in dbu.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbool.so")

GB_OK, GB_ERR_CAPACITY, GB_ERR_INVALID_BOX, GB_ERR_OOM, GB_ERR_TIMEOUT, GB_ERR_CUDA, GB_ERR_ARG, \
    GB_ERR_INTERNAL, GB_ERR_CORRUPT = range(9)
XOR, OR, AND, NOT, MERGE, SIZE = range(6)
OVERLAP = 7  # single-layer AND: area covered by at least two boxes of A

_ERRNAMES = {1: "CAPACITY", 2: "INVALID_BOX", 3: "OOM", 4: "TIMEOUT", 5: "CUDA", 6: "ARG", 7: "INTERNAL",
             8: "CORRUPT"}
# SNAP streams (box_codec.f90 / serialization.f90)
SNAP_BOXES_PER_CHUNK = 65536
COMPRESSION_METHOD_NONE, COMPRESSION_METHOD_SNAPPY = 0, 1


class GBError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("GB_ERR_%s (%d): %s" % (_ERRNAMES.get(code, "?"), code, msg))
        self.code = code


class c_box(ctypes.Structure):
    _fields_ = [("x1", ctypes.c_int32), ("y1", ctypes.c_int32), ("x2", ctypes.c_int32), ("y2", ctypes.c_int32)]


_lib = None


def lib():
    """Load libgbool.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libgbool.so is not built (run __graft_entry__.build()); "
                           "there is no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    P, i32, i64, u64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64
    pp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "gb_context_create": (ctypes.c_int, [ctypes.c_int, u64, pp]),
        "gb_context_destroy": (ctypes.c_int, [P]),
        "gb_set_stream": (ctypes.c_int, [P, P]),
        "gb_last_error": (ctypes.c_char_p, [P]),
        "gb_sync": (ctypes.c_int, [P, P]),
        "gb_clear_status": (None, [P]),
        "gb_arena_mark": (u64, [P]),
        "gb_arena_release": (ctypes.c_int, [P, u64]),
        "gb_set_capacity_factor": (ctypes.c_int, [P, ctypes.c_int]),
        "gb_set_tile_scratch": (ctypes.c_int, [P, u64]),
        "gb_layer_from_host": (ctypes.c_int, [P, P, u64, P, ctypes.c_int, pp]),
        "gb_layer_from_device": (ctypes.c_int, [P, P, u64, P, ctypes.c_int, pp]),
        "gb_layer_ncell": (ctypes.c_int, [P]),
        "gb_layer_count": (ctypes.c_int, [P, P, P, P]),
        "gb_layer_to_host": (ctypes.c_int, [P, P, P, u64, P, P]),
        "gb_layer_free": (None, [P, P]),
        "gb_op_bool": (ctypes.c_int, [P, ctypes.c_int, P, P, pp]),
        "gb_op_grow": (ctypes.c_int, [P, P, i32, i32, i32, i32, pp]),
        "gb_op_size": (ctypes.c_int, [P, P, i32, pp]),
        "gb_op_area": (ctypes.c_int, [P, P, P]),
        "gb_components": (ctypes.c_int, [P, P, u64, P, P]),
        "gb_morton_sort": (ctypes.c_int, [P, P, i64, ctypes.c_int, P, P]),
        "gb_canonical_sort": (ctypes.c_int, [P, P, i64]),
        "gb_um_to_dbu": (i32, [ctypes.c_double]),
        "PerformBoostPolygonOperation": (None, [P, ctypes.c_ulong, P, ctypes.c_ulong, P, P, ctypes.c_ulong,
                                                ctypes.c_long]),
        "PerformBoostPolygonMerge": (None, [P, ctypes.c_ulong, P, P]),
        "thrust_sort_boxes_direct": (None, [P, i64]),
        "thrust_sort_boxes_indirect": (None, [P, P, i64]),
        "device_event_sort": (None, [P, i64]),
        "gb_op1": (ctypes.c_int, [P, P, i32, P]),
        "gb_op1_host": (ctypes.c_int, [P, P, u64, P, ctypes.c_int, i32, P, P, P]),
        "gb_op1_host_digest": (ctypes.c_int, [P, P, u64, P, ctypes.c_int, i32, P, P, P, P]),
        "gb_layer_digest": (ctypes.c_int, [P, P, P]),
        "gb_radix_plan": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, i64, P, P]),
        "gb_op1_area": (ctypes.c_int, [P, P, i32, P, P]),
        "gb_graph_begin": (ctypes.c_int, [P]),
        "gb_graph_end": (ctypes.c_int, [P, pp]),
        "gb_graph_launch": (ctypes.c_int, [P, P]),
        "gb_graph_kernels": (i64, [P]),
        "gb_graph_destroy": (None, [P]),
        "gb_profile": (ctypes.c_int, [P, ctypes.c_int]),
        "gb_profile_read": (ctypes.c_int, [P, P, P, P, P]),
        "gb_launch_count": (i64, [P]),
        "gb_run_deck": (ctypes.c_int, [ctypes.c_char_p, P, u64, P]),
        "gb_debug_lookback_timeout": (ctypes.c_int, [P, ctypes.c_int]),
        "gb_radix_sort_device": (ctypes.c_int, [P, P, P, i64, ctypes.c_int, P, P]),
        "gb_radix_sort_device_cfg": (ctypes.c_int, [P, P, P, i64, ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int]),
        "gb_radix_autotune": (ctypes.c_int, [P, P, P, i64, ctypes.c_int, P, P, P]),
        "gb_radix_tuning_reset": (None, []),
        "gb_interactions": (ctypes.c_int, [P, P, u64, P, P, P]),
        "gb_certify_healing": (ctypes.c_int, [P, P, u64, P]),
        "gb_component_areas": (ctypes.c_int, [P, P, u64, P, u64, P]),
        "gb_morton_keys_device": (ctypes.c_int, [P, P, i64, P, P]),
        "gb_serve_create": (ctypes.c_int, [ctypes.c_int, u64, ctypes.c_int, u64, pp]),
        "gb_serve_add_layer": (ctypes.c_int, [P, P, u64, P]),
        "gb_serve_run": (ctypes.c_int, [P, P, ctypes.c_int, P, ctypes.c_int]),
        "gb_serve_result_boxes": (ctypes.c_int, [P, ctypes.c_int, P, u64, P]),
        "gb_serve_destroy": (None, [P]),
        "gb_bool_tile_noalloc": (ctypes.c_int, [ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int, P, i64, P, P, P]),
        "gb_set_grid": (ctypes.c_int, [P, ctypes.c_int]),
        "gb_get_grid": (ctypes.c_int, [P]),
        "gb_grid_autotune": (ctypes.c_int, [P, P, i32, P, P]),
        "gb_snap_max_bytes": (ctypes.c_int, [i64, P]),
        "gb_compress_boxes_to_stream": (ctypes.c_int, [P, P, i64, ctypes.c_int, P, i64, P, P]),
        "gb_decompress_stream_to_boxes": (ctypes.c_int, [P, P, P, i64, ctypes.c_int, P]),
        "gb_save_layer_to_snap": (ctypes.c_int, [P, ctypes.c_char_p, P, i64, ctypes.c_int, ctypes.c_int, P]),
        "gb_snap_file_info": (ctypes.c_int, [ctypes.c_char_p, P, P, P, P]),
        "gb_restore_snap_to_layer": (ctypes.c_int, [P, ctypes.c_char_p, P, i64, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _boxes(b):
    b = np.ascontiguousarray(b, dtype=np.int32).reshape(-1, 4)
    return b


class Layer:
    """A device-resident layer (raw boxes, or a binned operator result)."""

    def __init__(self, ctx, handle, ncell):
        self.ctx = ctx
        self.h = handle
        self.ncell = ncell

    def count(self):
        t = ctypes.c_int64()
        per = np.zeros(self.ncell, np.int64)
        self.ctx._chk(lib().gb_layer_count(self.ctx.h, self.h, ctypes.byref(t), per.ctypes.data))
        return int(t.value), per

    def digest(self):
        """Per-cell digest of the layer's strips (uint64, order-independent;
        gb_layer_digest)."""
        out = np.zeros(self.ncell, np.uint64)
        self.ctx._chk(lib().gb_layer_digest(self.ctx.h, self.h, out.ctypes.data))
        return out

    def to_numpy(self, with_cells=False):
        n = ctypes.c_uint64()
        L = lib()
        rc = L.gb_layer_to_host(self.ctx.h, self.h, None, 0, ctypes.byref(n), None)
        if rc not in (GB_OK, GB_ERR_CAPACITY):
            self.ctx._chk(rc)
        out = np.zeros((max(1, n.value), 4), np.int32)
        off = np.zeros(self.ncell + 1, np.int64)
        self.ctx._chk(L.gb_layer_to_host(self.ctx.h, self.h, out.ctypes.data, n.value, ctypes.byref(n),
                                         off.ctypes.data))
        out = out[:n.value]
        return (out, off) if with_cells else out

    def free(self):
        if self.h:
            lib().gb_layer_free(self.ctx.h, self.h)
            self.h = None


class Context:
    """A GPU context: stream, work arena, persistent-kernel resources."""

    def __init__(self, device=0, arena_bytes=0):
        h = ctypes.c_void_p()
        rc = lib().gb_context_create(device, arena_bytes, ctypes.byref(h))
        if rc != GB_OK:
            raise GBError(rc, "gb_context_create failed")
        self.h = h

    def close(self):
        if self.h:
            lib().gb_context_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, rc):
        if rc != GB_OK:
            msg = (lib().gb_last_error(self.h) or b"").decode()
            lib().gb_clear_status(self.h)  # the error is reported once, by this exception
            raise GBError(rc, msg)

    def sync(self):
        need = ctypes.c_int64()
        self._chk(lib().gb_sync(self.h, ctypes.byref(need)))

    def set_stream(self, stream_handle):
        self._chk(lib().gb_set_stream(self.h, ctypes.c_void_p(stream_handle)))

    def set_grid(self, g):
        """Tile grid of the operators: slab height 2^g dbu (10..16, default 16)."""
        self._chk(lib().gb_set_grid(self.h, g))

    @property
    def grid(self):
        return lib().gb_get_grid(self.h)

    def grid_autotune(self, P, amount=1):
        """Time the OP1 deck on layer P at tile grids 2^13..2^16 and keep the
        fastest on the context.  Returns (grid, {grid: ms or None})."""
        g = ctypes.c_int()
        ms = (ctypes.c_float * 4)()
        self._chk(lib().gb_grid_autotune(self.h, P.h, amount, ctypes.byref(g), ms))
        return g.value, {13 + i: (ms[i] if ms[i] > 0 else None) for i in range(4)}

    def mark(self):
        return lib().gb_arena_mark(self.h)

    def release(self, mark):
        self._chk(lib().gb_arena_release(self.h, mark))

    def layer(self, boxes, cell_offsets=None):
        b = _boxes(boxes)
        h = ctypes.c_void_p()
        if cell_offsets is None:
            self._chk(lib().gb_layer_from_host(self.h, b.ctypes.data, len(b), None, 1, ctypes.byref(h)))
            return Layer(self, h, 1)
        off = np.ascontiguousarray(cell_offsets, np.int64)
        self._chk(lib().gb_layer_from_host(self.h, b.ctypes.data, len(b), off.ctypes.data, len(off) - 1,
                                           ctypes.byref(h)))
        return Layer(self, h, len(off) - 1)

    def op(self, op, A, B=None):
        h = ctypes.c_void_p()
        self._chk(lib().gb_op_bool(self.h, op, A.h, B.h if B is not None else None, ctypes.byref(h)))
        return Layer(self, h, A.ncell)

    def grow(self, A, E, N, W, S):
        h = ctypes.c_void_p()
        self._chk(lib().gb_op_grow(self.h, A.h, E, N, W, S, ctypes.byref(h)))
        return Layer(self, h, A.ncell)

    def size(self, A, s):
        h = ctypes.c_void_p()
        self._chk(lib().gb_op_size(self.h, A.h, s, ctypes.byref(h)))
        return Layer(self, h, A.ncell)

    def area(self, A):
        out = np.zeros(A.ncell, np.int64)
        self._chk(lib().gb_op_area(self.h, A.h, out.ctypes.data))
        return out

    def components(self, boxes):
        b = _boxes(boxes)
        n = ctypes.c_int64()
        labels = np.zeros(len(b), np.int64)
        self._chk(lib().gb_components(self.h, b.ctypes.data, len(b), ctypes.byref(n), labels.ctypes.data))
        return int(n.value), labels

    def morton_sort(self, boxes):
        b = _boxes(boxes).copy()
        keys = np.zeros(len(b), np.uint64)
        perm = np.zeros(len(b), np.int64)
        self._chk(lib().gb_morton_sort(self.h, b.ctypes.data, len(b), 1, keys.ctypes.data, perm.ctypes.data))
        return b, keys, perm

    def op1(self, P, amount):
        """OP1 deck on layer P; returns the six result layers."""
        outs = (ctypes.c_void_p * 6)()
        self._chk(lib().gb_op1(self.h, P.h, amount, outs))
        return [Layer(self, ctypes.c_void_p(outs[i]), P.ncell) for i in range(6)]

    def op1_area(self, P, amount, area_ptr):
        """OP1 deck on layer P plus its union area per cell, written to the
        device int64 array at area_ptr; returns the six result layers."""
        outs = (ctypes.c_void_p * 6)()
        self._chk(lib().gb_op1_area(self.h, P.h, amount, outs, area_ptr))
        return [Layer(self, ctypes.c_void_p(outs[i]), P.ncell) for i in range(6)]

    def op1_host(self, boxes_ptr, n, offsets, amount, digests=False):
        """OP1 deck through host buffers (boxes_ptr: address of n int32x4
        boxes, e.g. pinned memory).  Returns (counts[ncell,6], area[ncell],
        assert_failures), plus digests[ncell,6] (uint64 per cell and result
        layer) when digests is true."""
        off = np.ascontiguousarray(offsets, np.int64)
        ncell = len(off) - 1
        counts = np.zeros((ncell, 6), np.int64)
        area = np.zeros(ncell, np.int64)
        fails = ctypes.c_int()
        if digests:
            dig = np.zeros((ncell, 6), np.uint64)
            self._chk(lib().gb_op1_host_digest(self.h, ctypes.c_void_p(boxes_ptr), n, off.ctypes.data, ncell, amount,
                                               counts.ctypes.data, area.ctypes.data, dig.ctypes.data,
                                               ctypes.byref(fails)))
            return counts, area, fails.value, dig
        self._chk(lib().gb_op1_host(self.h, ctypes.c_void_p(boxes_ptr), n, off.ctypes.data, ncell, amount,
                                    counts.ctypes.data, area.ctypes.data, ctypes.byref(fails)))
        return counts, area, fails.value

    def graph_begin(self):
        self._chk(lib().gb_graph_begin(self.h))

    def graph_end(self):
        g = ctypes.c_void_p()
        self._chk(lib().gb_graph_end(self.h, ctypes.byref(g)))
        return g

    def graph_launch(self, g):
        self._chk(lib().gb_graph_launch(self.h, g))

    def profile(self, on):
        self._chk(lib().gb_profile(self.h, 1 if on else 0))

    def profile_read(self):
        ms = ctypes.c_double()
        n, bi, bo = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._chk(lib().gb_profile_read(self.h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(bi),
                                        ctypes.byref(bo)))
        return ms.value, n.value, bi.value, bo.value

    def interactions(self, boxes):
        """(strict overlap pairs, singletons, singleton mask) of host boxes."""
        b = _boxes(boxes)
        p, s = ctypes.c_int64(), ctypes.c_int64()
        mask = np.zeros(len(b), np.uint8)
        self._chk(lib().gb_interactions(self.h, b.ctypes.data, len(b), ctypes.byref(p), ctypes.byref(s),
                                        mask.ctypes.data))
        return p.value, s.value, mask

    def certify_healing(self, boxes):
        b = _boxes(boxes)
        h = ctypes.c_int()
        self._chk(lib().gb_certify_healing(self.h, b.ctypes.data, len(b), ctypes.byref(h)))
        return bool(h.value)

    def component_areas(self, boxes):
        """Union area per component: [singleton area, component 1, ...]."""
        b = _boxes(boxes)
        nl = ctypes.c_int64()
        r = lib().gb_component_areas(self.h, b.ctypes.data, len(b), None, 0, ctypes.byref(nl))
        if r not in (GB_OK, GB_ERR_CAPACITY):
            self._chk(r)
        out = np.zeros(max(1, nl.value), np.int64)
        self._chk(lib().gb_component_areas(self.h, b.ctypes.data, len(b), out.ctypes.data, len(out),
                                           ctypes.byref(nl)))
        return out[:nl.value]

    def canonical_sort(self, boxes):
        b = _boxes(boxes).copy()
        self._chk(lib().gb_canonical_sort(self.h, b.ctypes.data, len(b)))
        return b

    def radix_sort_device(self, keys_ptr, vals_ptr, n, bits, keys_tmp, vals_tmp, passes=0, tile=0):
        """Sort n device (uint64 key, uint32 value) pairs in place by the low
        `bits` key bits (asynchronous on the context stream).  passes/tile 0:
        the tuned or default configuration.  Returns the pass count."""
        L = lib()
        if passes or tile:
            r = L.gb_radix_sort_device_cfg(self.h, keys_ptr, vals_ptr, n, bits, keys_tmp, vals_tmp, passes, tile)
        else:
            r = L.gb_radix_sort_device(self.h, keys_ptr, vals_ptr, n, bits, keys_tmp, vals_tmp)
        if r < 0:
            self._chk(-r)
        return r

    # ---- SNAP streams: box codec + Snappy per 65536-box chunk, .snap files
    def compress_boxes_to_stream(self, boxes, method=COMPRESSION_METHOD_SNAPPY):
        """CompressBoxesToStream on the device.  boxes: numpy (n, 4) int32 or
        a CUDA int32 tensor.  Returns [(num_boxes, raw_byte_size,
        compressed_size, data bytes)] per chunk."""
        import torch
        d = _device_boxes(boxes)
        n = d.shape[0]
        cap = ctypes.c_int64()
        self._chk(lib().gb_snap_max_bytes(n, ctypes.byref(cap)))
        out = torch.empty(max(cap.value, 16), dtype=torch.uint8, device=d.device)
        nch = (n + SNAP_BOXES_PER_CHUNK - 1) // SNAP_BOXES_PER_CHUNK
        meta = np.zeros(3 * max(nch, 1), np.int64)
        tot = ctypes.c_int64()
        torch.cuda.synchronize(d.device)
        self._chk(lib().gb_compress_boxes_to_stream(self.h, d.data_ptr(), n, method, out.data_ptr(), cap.value,
                                                    meta.ctypes.data, ctypes.byref(tot)))
        data = out[:tot.value].cpu().numpy().tobytes()
        chunks, at = [], 0
        for i in range(nch):
            nb, rn, cn = (int(v) for v in meta[3 * i:3 * i + 3])
            chunks.append((nb, rn, cn, data[at:at + cn]))
            at += cn
        return chunks

    def decompress_stream_to_boxes(self, chunks, method=COMPRESSION_METHOD_SNAPPY, as_tensor=False):
        """DecompressStreamToBoxes on the device: chunks as returned by
        compress_boxes_to_stream (or read from a .snap file)."""
        import torch
        n = sum(c[0] for c in chunks)
        meta = np.array([v for c in chunks for v in c[:3]] or [0], np.int64)
        data = b"".join(bytes(c[3]) for c in chunks)
        dd = torch.frombuffer(bytearray(data) or bytearray(16), dtype=torch.uint8).cuda()
        out = torch.empty((max(n, 1), 4), dtype=torch.int32, device=dd.device)
        torch.cuda.synchronize(dd.device)
        self._chk(lib().gb_decompress_stream_to_boxes(self.h, dd.data_ptr(), meta.ctypes.data, len(chunks), method,
                                                      out.data_ptr()))
        out = out[:n]
        return out if as_tensor else out.cpu().numpy()

    def save_layer_to_snap(self, path, boxes, method=COMPRESSION_METHOD_SNAPPY, layer_properties=0, pnum=None):
        """SaveLayerToSnap / SaveCompressedStreamToDisk: write boxes (numpy or
        CUDA tensor) as a .snap file; pnum (int64 per box) is stored when given."""
        import torch
        d = _device_boxes(boxes)
        pn = None if pnum is None else np.ascontiguousarray(pnum, np.int64)
        torch.cuda.synchronize(d.device)
        self._chk(lib().gb_save_layer_to_snap(self.h, os.fsencode(path), d.data_ptr(), d.shape[0], method,
                                              layer_properties, None if pn is None else pn.ctypes.data))

    def restore_snap_to_layer(self, path, as_tensor=False):
        """RestoreSnapToLayer: (boxes, layer_properties, method, pnum or None)."""
        import torch
        n, nch, meth, props = snap_file_info(path)
        out = torch.empty((max(n, 1), 4), dtype=torch.int32, device="cuda")
        pn = np.zeros(max(n, 1), np.int64) if props & 4 else None
        got = ctypes.c_int64()
        torch.cuda.synchronize()
        self._chk(lib().gb_restore_snap_to_layer(self.h, os.fsencode(path), out.data_ptr(), n, ctypes.byref(got),
                                                 None if pn is None else pn.ctypes.data))
        out = out[:n]
        return (out if as_tensor else out.cpu().numpy()), props, meth, (pn[:n] if pn is not None else None)

    def radix_autotune(self, keys_ptr, vals_ptr, n, bits):
        """Time the built sort configurations on a copy of the pairs; the
        fastest is used by later sorts of this size class.  Returns
        (passes, tile keys, ms)."""
        p, it, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        self._chk(lib().gb_radix_autotune(self.h, keys_ptr, vals_ptr, n, bits, ctypes.byref(p), ctypes.byref(it),
                                          ctypes.byref(ms)))
        return p.value, it.value, ms.value


def _device_boxes(boxes):
    import torch
    if isinstance(boxes, torch.Tensor):
        return boxes.to(device="cuda", dtype=torch.int32).contiguous().view(-1, 4)
    return torch.from_numpy(_boxes(boxes).copy()).cuda()


def snap_file_info(path):
    """(total boxes, chunks, compression method, layer properties) of a .snap file."""
    n, c = ctypes.c_int64(), ctypes.c_int64()
    m, p = ctypes.c_int(), ctypes.c_int()
    rc = lib().gb_snap_file_info(os.fsencode(path), ctypes.byref(n), ctypes.byref(c), ctypes.byref(m), ctypes.byref(p))
    if rc != GB_OK:
        raise GBError(rc, "gb_snap_file_info failed for %s" % path)
    return n.value, c.value, m.value, p.value


# ---- the reference's own FFI, called exactly as the Fortran layer calls it
def boost_polygon_operation(A, B, control, value=0):
    """PerformBoostPolygonOperation with the caller-side buffer convention of
    boost_polygon_apif.f90:59-71 (4*max(AN,BN), 10*max for AND)."""
    A, B = _boxes(A), _boxes(B)
    mx = max(len(A), len(B))
    cap = (10 if control == AND else 4) * mx
    out = np.zeros((max(cap, 1), 4), np.int32)
    n = ctypes.c_ulong()
    lib().PerformBoostPolygonOperation(A.ctypes.data, len(A), B.ctypes.data, len(B), out.ctypes.data,
                                       ctypes.byref(n), control, value)
    return out[:n.value]


def boost_polygon_merge(A):
    A = _boxes(A)
    out = np.zeros((max(2 * len(A), 1), 4), np.int32)
    n = ctypes.c_ulong()
    lib().PerformBoostPolygonMerge(A.ctypes.data, len(A), out.ctypes.data, ctypes.byref(n))
    return out[:n.value]


def sort_boxes_direct(boxes):
    b = _boxes(boxes).copy()
    lib().thrust_sort_boxes_direct(b.ctypes.data, len(b))
    return b


def sort_boxes_indirect(boxes):
    b = _boxes(boxes)
    idx = np.zeros(len(b), np.int64)
    lib().thrust_sort_boxes_indirect(b.ctypes.data, idx.ctypes.data, len(b))
    return idx


TRACKER_DTYPE = np.dtype([("X", np.int32), ("Y", np.int32), ("polygonNumber", np.int8), ("pad", np.int8, 3)])


def event_sort(trackers):
    t = np.ascontiguousarray(trackers, dtype=TRACKER_DTYPE).copy()
    lib().device_event_sort(t.ctypes.data, len(t))
    return t


REQ_SIZE, REQ_GROW = 5, 6
REQUEST_DTYPE = np.dtype([("op", np.int32), ("a", np.int32), ("b", np.int32), ("amount", np.int32),
                          ("arrival_s", np.float64)])
RESULT_DTYPE = np.dtype([("status", np.int32), ("pad", np.int32), ("count", np.int64), ("start_s", np.float64),
                         ("end_s", np.float64), ("latency_ms", np.float64)])


class Server:
    """Request loop over layers resident in HBM (gb_serve_*): continuous
    admission into concurrent slots under a device-memory budget."""

    def __init__(self, device=0, budget_bytes=120 << 30, slots=8, slot_arena_bytes=8 << 30):
        h = ctypes.c_void_p()
        rc = lib().gb_serve_create(device, budget_bytes, slots, slot_arena_bytes, ctypes.byref(h))
        if rc != GB_OK:
            raise GBError(rc, "gb_serve_create failed")
        self.h = h

    def add_layer(self, boxes):
        b = _boxes(boxes)
        i = ctypes.c_int()
        rc = lib().gb_serve_add_layer(self.h, b.ctypes.data, len(b), ctypes.byref(i))
        if rc != GB_OK:
            raise GBError(rc, "gb_serve_add_layer failed")
        return i.value

    def run(self, requests, keep_outputs=False):
        r = np.ascontiguousarray(requests, REQUEST_DTYPE)
        out = np.zeros(len(r), RESULT_DTYPE)
        rc = lib().gb_serve_run(self.h, r.ctypes.data, len(r), out.ctypes.data, 1 if keep_outputs else 0)
        if rc != GB_OK:
            raise GBError(rc, "gb_serve_run failed")
        return out

    def result_boxes(self, i):
        n = ctypes.c_uint64()
        lib().gb_serve_result_boxes(self.h, i, None, 0, ctypes.byref(n))
        out = np.zeros((max(1, n.value), 4), np.int32)
        lib().gb_serve_result_boxes(self.h, i, out.ctypes.data, n.value, ctypes.byref(n))
        return out[:n.value]

    def close(self):
        if self.h:
            lib().gb_serve_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def run_deck(path, log_cap=1 << 20):
    """Run a control deck on the GPU engine; returns (status, log, assert_failures)."""
    buf = ctypes.create_string_buffer(log_cap)
    fails = ctypes.c_int()
    rc = lib().gb_run_deck(os.fsencode(path), buf, log_cap, ctypes.byref(fails))
    return rc, buf.value.decode(errors="replace"), fails.value


def um_to_dbu(r):
    return int(lib().gb_um_to_dbu(float(r)))
