"""CPU FP64 oracle of the DL_POLY force/update path -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load this
package, as the reference results of the parity tests (or the timed CPU baseline); the
product never does.
"""
import ctypes
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.join(os.path.dirname(HERE), "dl-poly_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from dlpoly_gb300.binding import PathLib  # noqa: E402


def load(openmp: bool = False) -> PathLib:
    """Load the oracle library (building it first if it is missing)."""
    name = "liboracle_omp.so" if openmp else "liboracle.so"
    path = os.path.join(HERE, "_build", name)
    if not os.path.exists(path):
        from .build import build
        build()
    lib = ctypes.CDLL(path)
    pl = PathLib(lib, "orc_")
    lib.orc_set_threads.argtypes = [ctypes.c_int]
    lib.orc_set_threads.restype = ctypes.c_int
    return pl
