"""The C-ABI library loads and exports every entry point the header declares
(no compute calls: these run without a GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

import dlpoly_gb300 as gb
from dlpoly_gb300 import systems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_declares_the_path():
    names = gb.exported_symbols()
    for n in ("gb_init", "gb_upload_state", "gb_list_build", "gb_vnl_check", "gb_forces", "gb_spme", "gb_vv",
              "gb_md_run", "gb_download_state", "gb_finalize", "gb_strerror", "gb_mts_config"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(gb.LIB_PATH)
    missing = [n for n in gb.exported_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_strerror_codes():
    lib = ctypes.CDLL(gb.LIB_PATH)
    lib.gb_strerror.restype = ctypes.c_char_p
    lib.gb_strerror.argtypes = [ctypes.c_int]
    assert b"106" in lib.gb_strerror(106)
    assert b"SHAKE" in lib.gb_strerror(105)
    assert b"success" == lib.gb_strerror(0)


def test_calls_before_init_fail_cleanly():
    p = gb.load()
    u = np.zeros(1, np.int32)
    st = p.fn["vnl_check"](u.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
    assert st == -1  # GB_ERR_NOT_INIT


def test_params_struct_matches_header():
    # gb_params is 9+9 doubles then 3+1+... int32 fields: check the ctypes mirror size
    hdr = open(os.path.join(ROOT, "include", "gb300_dlpoly.h")).read()
    body = hdr[hdr.index("typedef struct gb_params"):hdr.index("} gb_params;")]
    ndouble = sum(int(m) if m else 1 for m in re.findall(r"double\s+\w+(?:\[(\d+)\])?;", body))
    nint = sum(int(m) if m else 1 for m in re.findall(r"int32_t\s+\w+(?:\[(\d+)\])?;", body))
    raw = 8 * ndouble + 4 * nint
    assert ctypes.sizeof(gb.GbParams) == (raw + 7) // 8 * 8  # C pads to the double alignment


def test_system_generators():
    s = systems.nacl_melt(16)
    assert s.natms == 4096 and abs(s.chge.sum()) < 1e-12
    assert s.cell[0] == pytest.approx(45.12)
    assert s.kmax == (48, 48, 48)
    w = systems.spce_water(8)
    assert w.natms == 1536 and abs(w.chge.sum()) < 1e-9
    dens = w.weight.sum() / 0.6022140857 / w.volume()
    assert dens == pytest.approx(1.0, rel=1e-6)
    # initial velocities satisfy the bond constraints (d . dv = 0)
    lc = w.listcon.reshape(-1, 3)
    X = np.stack([w.x, w.y, w.z], 1)
    V = np.stack([w.vx, w.vy, w.vz], 1)
    d = X[lc[:, 1] - 1] - X[lc[:, 2] - 1]
    dv = V[lc[:, 1] - 1] - V[lc[:, 2] - 1]
    assert np.abs((d * dv).sum(1)).max() < 1e-10
