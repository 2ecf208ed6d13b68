"""gb_kinstress_noalloc: the kinetic stress for callers that cannot allocate
device memory (their device memory belongs to a pool they do not control, or
they must not allocate once a run is under way).

The entry point is called through the C-ABI on device buffers the test owns,
twice in a row on two successive MD steps, and compared with the kinetic
stress the existing entry point (gb_md_run -> gb_vv stage 2, kinstress)
returns for the same velocities.  This file is named so pytest collects it
last.
"""
import ctypes

import numpy as np
import pytest

from dlpoly_gb300 import systems

pytestmark = pytest.mark.gpu

REL = 1e-10  # the FP64 tolerance of the parity tests (summation order differs)


def _bind(lib):
    f = lib.gb_kinstress_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_kinstress_noalloc_matches_gb_vv(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    f = _bind(gpu_lib.lib)
    s = systems.spce_water(8)
    s.lfrzn = s.lfrzn.copy()
    gpu_lib.init(s)
    gpu_lib.start()
    dev = torch.device("cuda", 0)
    w = torch.tensor(s.weight, dtype=torch.float64, device=dev)
    fr = torch.tensor(s.lfrzn, dtype=torch.int32, device=dev)
    out = torch.full((9,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(2):  # two calls in a row, on two successive steps
        st = gpu_lib.md_vv(1)[0]
        expect = np.array(st.strkin[:])
        d = gpu_lib.download()
        vx = torch.tensor(d["vx"], dtype=torch.float64, device=dev)
        vy = torch.tensor(d["vy"], dtype=torch.float64, device=dev)
        vz = torch.tensor(d["vz"], dtype=torch.float64, device=dev)
        rc = f(vx.data_ptr(), vy.data_ptr(), vz.data_ptr(), w.data_ptr(), fr.data_ptr(), s.natms, out.data_ptr(),
               ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        stream.synchronize()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.abs(got - expect).max() <= REL * np.abs(expect).max()
        out.fill_(float("nan"))


def _kin_numpy(d, w, frozen=None):
    """kinstress (kinetics.F90:218-262) in numpy: atoms with lfrzn != 0 are left out."""
    v = np.stack([d["vx"], d["vy"], d["vz"]], 1)
    m = w.copy()
    if frozen is not None:
        m = np.where(frozen != 0, 0.0, m)
    return np.einsum("i,ia,ib->ab", m, v, v).reshape(9)


def test_kinstress_noalloc_frozen_atoms_and_edge_sizes(gpu_lib):
    """The lfrzn != 0 branch (some atoms frozen), lfrzn = NULL (no frozen atoms) and n = 0."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device visible to torch")
    f = _bind(gpu_lib.lib)
    s = systems.nacl_melt(16)
    s.lfrzn = np.zeros(s.natms, np.int32)
    s.lfrzn[::97] = 1
    gpu_lib.init(s)
    gpu_lib.start()
    ref = gpu_lib.nve_0_vv(2)["strkin"]  # gb_vv stage 2: kinstress of the free atoms
    d = gpu_lib.download()
    dev = torch.device("cuda", 0)
    vx, vy, vz = (torch.tensor(d[k], dtype=torch.float64, device=dev) for k in ("vx", "vy", "vz"))
    w = torch.tensor(s.weight, dtype=torch.float64, device=dev)
    fr = torch.tensor(s.lfrzn, dtype=torch.int32, device=dev)
    out = torch.full((9,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    expect_free = _kin_numpy(d, s.weight, s.lfrzn)
    expect_all = _kin_numpy(d, s.weight)
    # the frozen atoms carry velocity, so leaving them out changes the tensor
    assert np.abs(expect_all - expect_free).max() > 1e-6 * np.abs(expect_all).max()
    assert f(vx.data_ptr(), vy.data_ptr(), vz.data_ptr(), w.data_ptr(), fr.data_ptr(), s.natms, out.data_ptr(), sp) == 0
    stream.synchronize()
    got = out.cpu().numpy()
    assert np.abs(got - ref).max() <= REL * np.abs(ref).max()
    assert np.abs(got - expect_free).max() <= REL * np.abs(expect_free).max()
    # lfrzn = NULL: every atom counts
    out.fill_(float("nan"))
    assert f(vx.data_ptr(), vy.data_ptr(), vz.data_ptr(), w.data_ptr(), None, s.natms, out.data_ptr(), sp) == 0
    stream.synchronize()
    got = out.cpu().numpy()
    assert np.abs(got - expect_all).max() <= REL * np.abs(expect_all).max()
    # n = 0: an all-zero tensor, the array pointers are not read
    out.fill_(float("nan"))
    assert f(vx.data_ptr(), vy.data_ptr(), vz.data_ptr(), w.data_ptr(), None, 0, out.data_ptr(), sp) == 0
    stream.synchronize()
    assert np.array_equal(out.cpu().numpy(), np.zeros(9))


def test_kinstress_noalloc_rejects_too_many_atoms(gpu_lib):
    f = _bind(gpu_lib.lib)
    # nothing is launched for a size beyond the fixed scratch: pointers are never read
    dummy = ctypes.c_void_p(16)
    rc = f(dummy, dummy, dummy, dummy, None, 1 << 21, dummy, None)
    assert rc == -6
