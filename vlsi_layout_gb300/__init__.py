"""GB300-native engine for the Manhattan box-Boolean hot path of MAGPARSER.

The compute lives in libgbool.so (hand-written sm_103a CUDA behind a C-ABI,
include/gbool.h); `engine` is the ctypes binding, including the control-deck
runner `engine.run_deck` (gb_run_deck).
"""
from .engine import Context, Layer, GBError, XOR, OR, AND, NOT, MERGE, SIZE  # noqa: F401
