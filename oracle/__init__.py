"""Test oracle for the ALBATROS baseband path.

TEST INFRASTRUCTURE: only tests/, ``__graft_entry__.smoke()`` and the
cpu_baseline / reference legs of ``bench.py`` import this package, and only as
the checker or the timed CPU baseline; the product package never does.

- ``pfb_oracle``: FP64 NumPy restatement (window, matft, filter, IPFB, PFB,
  all-antenna correlator, streaming chain).
- ``c_oracle()``: ctypes handle on ``liboracle.so`` built from
  ``albatros_oracle.c`` (integer unpack / sortpols / correlators, exact int64).
- ``ref_libs()``: the reference's own C files compiled into ``_ref/`` by
  ``build.py`` when the reference sources are present (this container only).
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
_c = None


def c_oracle():
    """Load liboracle.so (built by oracle/build.py) with argtypes set."""
    global _c
    if _c is not None:
        return _c
    path = os.path.join(HERE, "liboracle.so")
    if not os.path.exists(path):
        from . import build as _b
        _b.build_oracle()
    lib = ctypes.CDLL(path)
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    sig = {
        "or_unpack_4bit_float": [P, P, P, I64, I64, P, I64, I64],
        "or_unpack_4bit_float_mt": [P, P, P, I64, I64, P, I64, I64, I],
        "or_unpack_1bit_float": [P, P, P, I64, I64, I64, I64, I64],
        "or_sortpols": [P, P, P, I64, I64, I64, I64, I, I64, I64],
        "or_hist_4bit": [P, P, I64, I64, I64, I64, I],
        "or_hist_1bit": [P, P, I64, I64, I64, I64, I],
        "or_avg_xcorr_4bit": [P, P, P, P, I64, I64],
        "or_avg_xcorr_4bit_2ant": [P, P, P, P, P, P, I64, I64, I64, I64, I64],
        "or_avg_xcorr_1bit": [P, P, P, P, I64, I64, I64],
        "or_avg_xcorr_1bit_vanvleck": [P, P, P, P, P, P, I64, I64, I64],
        "or_avg_xcorr_1bit_vanvleck_2ant": [P, P, P, P, P, P, P, P, I64, I64, I64, I64, I64, I64],
        "or_xcorr_all_ant_4bit": [P, I64, I64, I64, I64, I64, P, I64, P, P, I],
    }
    for name, args in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = I64 if name.endswith("_2ant") else None
    _c = lib
    return lib


def ref_libs():
    """(unpacking, correlations_cpu) CDLLs of the reference's own C, or None."""
    up = os.path.join(HERE, "_ref", "lib_unpacking.so")
    co = os.path.join(HERE, "_ref", "lib_correlations_cpu.so")
    if not (os.path.exists(up) and os.path.exists(co)):
        return None
    try:
        return ctypes.CDLL(up), ctypes.CDLL(co)
    except OSError:
        return None
