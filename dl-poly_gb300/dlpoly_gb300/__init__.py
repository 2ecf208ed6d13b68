"""GB300 (sm_103a) implementation of DL_POLY's per-timestep force and update path.

`load()` returns a `PathLib` bound to libdlpoly_gb300.so (the C-ABI declared in
include/gb300_dlpoly.h).  There is no CPU fallback: if the library is missing
or no CUDA device is present, the calls fail with an error.
"""
from __future__ import annotations

import ctypes
import os

from . import systems
from .binding import PathError, PathLib, stats_to_dict
from .systems import GbParams, GbStepStats, System

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdlpoly_gb300.so")

GB_FP64 = 0
GB_MIXED = 1

_lib = None


def load() -> PathLib:
    """Load libdlpoly_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it first (dlpoly_gb300.build.build())")
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.gb_kernel_launches.restype = ctypes.c_int64
        _lib.gb_set_precision.argtypes = [ctypes.c_int]
        _lib.gb_set_precision.restype = ctypes.c_int
        _lib.gb_last_timings.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        _lib.gb_last_timings.restype = ctypes.c_int
        _lib.gb_mts_config.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_int]
        _lib.gb_mts_config.restype = ctypes.c_int
    return PathLib(_lib, "gb_")


def exported_symbols() -> list[str]:
    """Names of every entry point declared in include/gb300_dlpoly.h."""
    import re

    hdr = os.path.join(os.path.dirname(os.path.dirname(HERE)), "include", "gb300_dlpoly.h")
    txt = open(hdr).read()
    return sorted(set(re.findall(r"^\s*(?:int|void|const char\*|int64_t)\s+(gb_\w+)\s*\(", txt, re.M)))


__all__ = ["load", "PathLib", "PathError", "System", "GbParams", "GbStepStats", "systems", "stats_to_dict",
           "GB_FP64", "GB_MIXED", "exported_symbols", "LIB_PATH"]
