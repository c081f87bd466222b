"""Build libgbool.so (the engine and its C-ABI) in-tree for sm_103a.

Each .cu translation unit is compiled by nvcc in parallel into _build/, then
linked into vlsi_layout_gb300/libgbool.so.  Nothing is installed.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgbool.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["gb_bin.cu", "gb_tile.cu", "gb_uf.cu", "gb_radix.cu", "gb_api.cu", "gb_deck.cu",
           "gb_deckrun.cu", "gb_serve.cu", "gb_snap.cu"]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _compile(src, verbose=False):
    s = os.path.join(CSRC, src)
    o = os.path.join(BUILD, src.replace(".cu", ".o"))
    deps = [s] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "gbool.h"))
    if os.path.exists(o) and all(os.path.getmtime(o) >= os.path.getmtime(d) for d in deps):
        return o
    cmd = [_nvcc()] + _flags() + (["-Xptxas", "-v"] if verbose else []) + ["-c", s, "-o", o]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    if verbose:
        sys.stderr.write(r.stderr)
    return o


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
