"""CPU tests of the FP64 oracle: the reference's own known answers, physics
invariants and the committed golden fixtures (no GPU needed)."""
import ctypes
import math
import os

import numpy as np
import pytest

from dlpoly_gb300 import systems

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
R4PIE0 = 138935.4835


def test_lj_known_answers(oracle_lib):
    """source/unit_tests/test_vdw.F90:46-59, entries 1 (12-6, a=1 b=2) and 2 (LJ eps=1 sigma=2) at r=1."""
    f = oracle_lib.lib.orc_lj_kat
    f.argtypes = [ctypes.c_double] * 3 + [ctypes.POINTER(ctypes.c_double)] * 2
    e, gmm = ctypes.c_double(), ctypes.c_double()
    f(1.0, 2.0, 1.0, ctypes.byref(e), ctypes.byref(gmm))
    assert e.value == 16128.0
    assert -gmm.value * 1.0 ** 2 == -195072.0  # virial = -gamma r^2
    # 12-6 with a=1, b=2 is LJ with sigma^6 = a/b, eps = b^2/(4a)
    f(1.0, 0.5 ** (1.0 / 6.0), 1.0, ctypes.byref(e), ctypes.byref(gmm))
    assert e.value == pytest.approx(-1.0, rel=1e-14)
    assert gmm.value == pytest.approx(0.0, abs=1e-12)


def test_lj_kat_through_pair_loop(oracle_lib):
    """The same known answer through link_cell_pairs + the direct vdW pair loop."""
    s = systems.lj_pair(eps=1.0, sigma=2.0, r=1.0)
    oracle_lib.init(s)
    oracle_lib.relocate()
    oracle_lib.link_cell_pairs()
    e, _ = oracle_lib.real_space_forces()
    assert e["engvdw"] == pytest.approx(16128.0, rel=1e-14)
    assert e["virvdw"] == pytest.approx(-195072.0, rel=1e-14)
    d = oracle_lib.download()
    # force on atom 1 along +x (repulsive), equal and opposite on atom 2
    assert d["fx"][1] == pytest.approx(195072.0, rel=1e-14)
    assert d["fx"][0] == pytest.approx(-195072.0, rel=1e-14)


def test_madelung_rock_salt(oracle_lib):
    """Perfect rock-salt lattice: Coulomb energy per ion = -M e^2 / (2 a), M = 1.747565."""
    s = systems.nacl_melt(16, jitter=0.0)
    oracle_lib.init(s)
    oracle_lib.relocate()
    oracle_lib.link_cell_pairs(want_list=False)
    e, _ = oracle_lib.two_body_forces()
    coul = e["engcpe_rc"] + e["engcpe_rl"] + e["engcpe_ex"]
    expect = -1.747564594633 * R4PIE0 / (2.0 * 2.82) * s.natms
    # the reference's erfc is the 5-term Abramowitz-Stegun fit (numerics.F90:3647,
    # |error| <= 1.5e-7), which biases the real-space sum at the 1e-5 level
    assert coul == pytest.approx(expect, rel=3e-5)
    d = oracle_lib.download()
    F = np.stack([d["fx"], d["fy"], d["fz"]], 1)
    # forces vanish at the lattice sites up to the LJ part (which is symmetric too)
    assert np.abs(F).max() < 1e-3 * R4PIE0 / 2.82 ** 2


def _total_energy(o, s):
    o.upload(s.x, s.y, s.z, s.vx, s.vy, s.vz)
    o.relocate()
    o.link_cell_pairs(want_list=False)
    e, _ = o.two_body_forces()
    return e["engcpe_rc"] + e["engcpe_rl"] + e["engcpe_ex"] + e["engvdw"]


def test_force_is_minus_gradient(oracle_lib):
    """Central differences of the total potential reproduce the forces."""
    s = systems.nacl_melt(16)
    s.vdw_direct = 1  # analytic vdW so energy and force are exact derivatives
    oracle_lib.init(s)
    _total_energy(oracle_lib, s)
    d = oracle_lib.download()
    F = np.stack([d["fx"], d["fy"], d["fz"]], 1)
    h = 1e-4
    rng = np.random.default_rng(3)
    for i in rng.choice(s.natms, 3, replace=False):
        for c, arr in enumerate(("x", "y", "z")):
            a = getattr(s, arr)
            a0 = a[i]
            a[i] = a0 + h
            ep = _total_energy(oracle_lib, s)
            a[i] = a0 - h
            em = _total_energy(oracle_lib, s)
            a[i] = a0
            fd = -(ep - em) / (2 * h)
            # tabulated erfc: interpolation consistency ~1e-6 of the force scale
            assert fd == pytest.approx(F[i, c], abs=2e-5 * np.abs(F).max())


def test_ewald_alpha_invariance(oracle_lib):
    """Total Coulomb energy does not depend on the Ewald splitting parameter."""
    out = []
    for alpha, k in ((0.26505830360350674, 48), (0.30, 64)):
        s = systems.nacl_melt(16)
        s.alpha = alpha
        s.kmax = (k, k, k)
        oracle_lib.init(s)
        oracle_lib.relocate()
        oracle_lib.link_cell_pairs(want_list=False)
        e, _ = oracle_lib.two_body_forces()
        out.append(e["engcpe_rc"] + e["engcpe_rl"])
    assert out[0] == pytest.approx(out[1], rel=2e-6)


def test_bspline_partition_of_unity(oracle_lib):
    f = oracle_lib.lib.orc_splines
    f.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    for p in (4, 6, 8, 10):
        buf = (ctypes.c_double * (3 * p))()
        for u in (10.0, 10.25, 11.5, 12.999):
            f(u, p, buf)
            v = np.array(buf[:])
            assert v[:p].sum() == pytest.approx(1.0, abs=1e-14)
            assert v[p:2 * p].sum() == pytest.approx(0.0, abs=1e-13)
            assert v[2 * p:].sum() == pytest.approx(0.0, abs=1e-12)
            assert (v[:p] >= -1e-15).all()


@pytest.mark.parametrize("name,make", [("nacl_4096", lambda: systems.nacl_melt(16)),
                                       ("water_1536", lambda: systems.spce_water(8))])
def test_oracle_matches_golden(oracle_lib, name, make):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    s = make()
    oracle_lib.init(s)
    oracle_lib.relocate()
    lst = oracle_lib.link_cell_pairs()
    assert np.array_equal(lst[:, 3], g["list_count"])
    assert np.array_equal(lst[:, 2], g["list_excl_end"])
    e, st = oracle_lib.two_body_forces()
    d = oracle_lib.download()
    F = np.stack([d["fx"], d["fy"], d["fz"]], 1)
    rms = np.sqrt((g["f0"] ** 2).sum(1).mean())
    assert np.abs(F - g["f0"]).max() / rms < 1e-11
    for k, v in zip(g["eng_keys"], g["eng0"]):
        assert e[str(k)] == pytest.approx(v, rel=1e-11, abs=1e-6)
    stats = oracle_lib.md_vv(5)
    d = oracle_lib.download()
    X = np.stack([d["x"], d["y"], d["z"]], 1)
    assert np.abs(X - g["x5"]).max() < 1e-9
    assert [s_.shake_iters for s_ in stats] == list(g["shake_iters"])


def test_nve_energy_conservation(oracle_lib):
    s = systems.nacl_melt(16)
    oracle_lib.init(s)
    e, _ = oracle_lib.start()
    stats = oracle_lib.md_vv(40)
    tot = np.array([st.engke + st.engcpe_rc + st.engcpe_rl + st.engcpe_ex + st.engvdw for st in stats])
    ke = np.mean([st.engke for st in stats])
    # fluctuation of the conserved energy small compared with the kinetic energy
    assert np.std(tot) < 2e-3 * ke
    assert any(st.list_rebuilt for st in stats)


def test_shake_keeps_bonds(oracle_lib):
    s = systems.spce_water(8)
    oracle_lib.init(s)
    oracle_lib.start()
    oracle_lib.md_vv(5)
    d = oracle_lib.download()
    X = np.stack([d["x"], d["y"], d["z"]], 1)
    lc = s.listcon.reshape(-1, 3)
    dv = X[lc[:, 1] - 1] - X[lc[:, 2] - 1]
    L = s.cell[0]
    dv -= L * np.round(dv / L)
    dist = np.linalg.norm(dv, axis=1)
    target = s.prmcon[lc[:, 0] - 1]
    # converged to |d^2 - d0^2|/2 < tol * d0
    assert np.max(np.abs(dist ** 2 - target ** 2) / 2 / target) < s.shake_tol * 1.0001


def test_list_overflow_reports_needed_size(oracle_lib):
    s = systems.nacl_melt(16)
    oracle_lib.init(s, max_list=50)
    oracle_lib.relocate()
    st, need = oracle_lib.list_build_status()
    assert st == 106
    assert need > 50
