"""Generate tests/golden/golden.json from the reference's own in-repo fixtures.

Reads the KLBin fixtures (raw little-endian int32 x4 records, the format of
kldata.f90:14-72) of the mounted reference and records, per fixture: the
boxes, and the results of the reference's own compiled CPU Morton sort
(gpu_morton.cu, #ifndef USE_GPU branch, built by oracle/Makefile into
oracle/_ref) next to the oracle's results.  Run from the repository root:
    python tests/golden/make_golden.py
"""
import ctypes
import glob
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

REF = "/root/reference/src"


def main():
    O.build()
    ref = O.ref_sort_lib()
    files = sorted(glob.glob(os.path.join(REF, "SEDFXTP1_DATA", "*.bin"))) + \
        [os.path.join(REF, "square_L68_D20.bin"), os.path.join(REF, "square.bin_L68_D20.bin")]
    out = {"source": "reference KLBin fixtures (src/SEDFXTP1_DATA/*.bin, src/square*_L68_D20.bin)",
           "fixtures": {}}
    for f in files:
        b = np.fromfile(f, dtype="<i4").reshape(-1, 4)
        name = os.path.relpath(f, REF)
        rec = {"boxes": b.tolist()}
        if ref is not None and len(b):
            s = np.ascontiguousarray(b.copy())
            ref.thrust_sort_boxes_direct(s.ctypes.data, len(s))
            rec["ref_morton_sorted_keys"] = [int(k) for k in O.morton_keys(s)]
            idx = np.zeros(len(b), np.int64)
            ref.thrust_sort_boxes_indirect(np.ascontiguousarray(b).ctypes.data, idx.ctypes.data, len(b))
            rec["ref_morton_indirect_keys"] = [int(k) for k in O.morton_keys(b[idx - 1])]
        rec["sum_area"] = O.area_of(b) if len(b) else 0
        rec["union_area"] = O.union_area(b)
        rec["merge"] = O.merge(b).tolist() if len(b) else []
        rec["components"] = O.components(b)[0] if len(b) else 0
        out["fixtures"][name] = rec
    path = os.path.join(ROOT, "tests", "golden", "golden.json")
    with open(path, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote", path, len(out["fixtures"]), "fixtures")


if __name__ == "__main__":
    main()
