"""Generate tests/golden/golden.json from the reference's own in-repo fixtures.

Reads the KLBin fixtures (raw little-endian int32 x4 records, the format of
kldata.f90:14-72) of the reference sources and records, per fixture:

* from the REFERENCE's own compiled CPU code (gpu_morton.cu and
  event_sorter.cu, their #ifndef USE_GPU branch, built by oracle/Makefile into
  oracle/_ref): the Morton order of thrust_sort_boxes_direct /
  thrust_sort_boxes_indirect, and the tracker order of cpp_std_sort_trackers
  on the fixture's corner tokens (four per box with the signs of
  generate_trackers, polygon_fracture.f90:767-803);
* from the ORACLE (this repository's CPU restatement): the healed strips, the
  union area and the component count, as regression values;
* plain arithmetic: the sum of box areas.

The "provenance" field of the file says which keys are which.  It also records
a seeded 200000-tracker set (numpy PCG64) sorted by cpp_std_sort_trackers, as
a SHA-256 of the canonical (X, Y, polygonNumber) order: std::sort is not
stable, so payloads are compared as a multiset per key.

Run from the repository root with the reference sources at $GB_REFERENCE_SRC
(default: the mounted reference's src/ directory):
    GB_REFERENCE_SRC=/path/to/VLSI_LAYOUT/src python tests/golden/make_golden.py
"""
import glob
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

REF = os.environ.get("GB_REFERENCE_SRC", "/root/reference/src")
sys.path.insert(0, os.path.join(ROOT, "tests"))
from trackers import canonical_digest, corner_trackers, seeded_trackers  # noqa: E402


def main():
    O.build()
    ref = O.ref_sort_lib()
    if ref is None:
        sys.exit("the reference's CPU sort helpers were not built (oracle/Makefile ref): set GB_REFERENCE_SRC")
    files = sorted(glob.glob(os.path.join(REF, "SEDFXTP1_DATA", "*.bin"))) + \
        [os.path.join(REF, "square_L68_D20.bin"), os.path.join(REF, "square.bin_L68_D20.bin")]
    out = {"source": "reference KLBin fixtures (src/SEDFXTP1_DATA/*.bin, src/square*_L68_D20.bin)",
           "provenance": {
               "reference": ["ref_morton_sorted_keys", "ref_morton_indirect_keys", "ref_sorted_trackers",
                             "seeded_trackers.sha256"],
               "oracle": ["merge", "union_area", "components"],
               "arithmetic": ["sum_area"],
               "input": ["boxes", "seeded_trackers.n", "seeded_trackers.seed"]},
           "fixtures": {}}
    for f in files:
        b = np.fromfile(f, dtype="<i4").reshape(-1, 4)
        name = os.path.relpath(f, REF)
        rec = {"boxes": b.tolist()}
        if len(b):
            s = np.ascontiguousarray(b.copy())
            ref.thrust_sort_boxes_direct(s.ctypes.data, len(s))
            rec["ref_morton_sorted_keys"] = [int(k) for k in O.morton_keys(s)]
            idx = np.zeros(len(b), np.int64)
            ref.thrust_sort_boxes_indirect(np.ascontiguousarray(b).ctypes.data, idx.ctypes.data, len(b))
            rec["ref_morton_indirect_keys"] = [int(k) for k in O.morton_keys(b[idx - 1])]
            t = corner_trackers(b)
            ref.cpp_std_sort_trackers(t.ctypes.data, len(t))
            rec["ref_sorted_trackers"] = np.stack([t["X"], t["Y"], t["polygonNumber"].astype(np.int32)], 1).tolist()
        rec["sum_area"] = O.area_of(b) if len(b) else 0
        rec["union_area"] = O.union_area(b)
        rec["merge"] = O.merge(b).tolist() if len(b) else []
        rec["components"] = O.components(b)[0] if len(b) else 0
        out["fixtures"][name] = rec
    t = seeded_trackers()
    ref.cpp_std_sort_trackers(t.ctypes.data, len(t))
    out["seeded_trackers"] = {"n": len(t), "seed": 17, "x_range": [-50000, 50000], "y_range": [-50000, 50000],
                              "sha256": canonical_digest(t)}
    path = os.path.join(ROOT, "tests", "golden", "golden.json")
    with open(path, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote", path, len(out["fixtures"]), "fixtures")


if __name__ == "__main__":
    main()
