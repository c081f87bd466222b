"""Generate tests/golden/snap_golden.json: SNAP streams (box codec + Snappy)
for the reference's KLBin fixtures and for seeded synthetic layers.

The reference's own check of this path (generate_bin.f90:182-262,
TestSnappyCompression / TestSnappyDecompression) loads a KLBin layer, Morton
sorts it, compresses it with CompressBoxesToStream and restores it.  Here
each layer is Morton sorted (device key form of gpu_morton.cu, stable) and,
per 65536-box chunk, recorded as
  * the box codec's bytes (oracle restatement of box_codec.f90:616-698), and
  * the Snappy library's compression of those bytes (the library the
    reference links, reached through pyarrow's bundled copy), so that the
    decoders are checked against a compressor that is not this project's.
The KLBin fixtures are stored as boxes; the synthetic layers (tests/gen.py,
seeded) as their generator arguments and a SHA-256 of the boxes.  Run from
the repository root, where pyarrow is installed:
    python tests/golden/make_snap_golden.py
"""
import base64
import glob
import hashlib
import json
import os
import sys

import numpy as np
import pyarrow as pa

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import oracle as O  # noqa: E402
from gen import macro_arrays, stdcell_layers  # noqa: E402

REF = os.environ.get("GB_REFERENCE_SRC", "/root/reference/src")  # the reference sources


def morton_sorted(A):
    return A[np.argsort(O.morton_keys_np(A), kind="stable")]


def chunks_of(A):
    out = []
    for c0 in range(0, len(A), O.BOXES_PER_CHUNK):
        part = A[c0:c0 + O.BOXES_PER_CHUNK]
        raw = O.codec_encode_chunk(part)
        lib = pa.compress(raw, codec="snappy", asbytes=True)
        out.append({"num_boxes": len(part), "raw_byte_size": len(raw),
                    "raw_sha256": hashlib.sha256(raw).hexdigest(),
                    "snappy_library": base64.b64encode(lib).decode()})
    return out


def synthetic():
    sc = stdcell_layers(3000, seed=11)
    rows = np.concatenate([sc[k] for k in ("poly", "met1", "met2", "li1", "contact")])
    macros = macro_arrays(nmacro=20, seed=5)  # 81920 boxes: two chunks, the second ragged
    return {"stdcell_layers_3000": ("stdcell_layers", {"n_per_layer": 3000, "seed": 11}, rows),
            "macro_arrays_20": ("macro_arrays", {"nmacro": 20, "seed": 5}, macros)}


def main():
    O.build()
    out = {"source": "reference KLBin fixtures (src/SEDFXTP1_DATA/*.bin) and seeded tests/gen.py layers; "
                     "Snappy bytes from the Snappy library via pyarrow %s" % pa.__version__,
           "codec_known_answer": {
               # box_codec.f90:616-698 by hand: (0,0,10,10) square, new width 10 -> 0x13 0x0a;
               # (5,0,15,20) dx 5, width 10 unchanged, new height 20 -> 0x2c 0x0a 0x14;
               # (5,-3,12,17) dy -3, new width 7, height 20 unchanged -> 0x43 0x05 0x07;
               # (0,0,10,20) dx -5, dy 3, width 10 seen (index 1), height unchanged -> 0x61 0x09 0x06 0x01 0x00
               "boxes": [[0, 0, 10, 10], [5, 0, 15, 20], [5, -3, 12, 17], [0, 0, 10, 20]],
               "bytes_hex": "130a2c0a144305076109060100"},
           "fixtures": {}, "synthetic": {}}
    kat = np.array(out["codec_known_answer"]["boxes"], np.int32)
    assert O.codec_encode_chunk(kat).hex() == out["codec_known_answer"]["bytes_hex"]
    files = sorted(glob.glob(os.path.join(REF, "SEDFXTP1_DATA", "*.bin")))
    allb = []
    for f in files:
        b = np.fromfile(f, dtype="<i4").reshape(-1, 4)
        allb.append(b)
        A = morton_sorted(b)
        out["fixtures"][os.path.relpath(f, REF)] = {"boxes": A.tolist(), "chunks": chunks_of(A)}
    A = morton_sorted(np.concatenate(allb))
    out["fixtures"]["SEDFXTP1_DATA (all layers)"] = {"boxes": A.tolist(), "chunks": chunks_of(A)}
    for name, (fn, kw, B) in synthetic().items():
        A = morton_sorted(B)
        out["synthetic"][name] = {"generator": fn, "args": kw,
                                  "sha256": hashlib.sha256(A.astype("<i4").tobytes()).hexdigest(),
                                  "n": len(A), "chunks": chunks_of(A)}
    path = os.path.join(ROOT, "tests", "golden", "snap_golden.json")
    with open(path, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
