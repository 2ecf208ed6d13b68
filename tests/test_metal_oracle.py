"""Tabulated EAM metals in the oracle (CPU): known answers from polynomial tables,
for which the reference's table derivative and three-point interpolation are exact;
forces against finite differences of the energy; the error statuses 506 / 507."""
import numpy as np
import pytest

from dlpoly_gb300 import systems


def two_atoms(r, ntypes=1, box=30.0):
    n = 2
    cell = np.array([box, 0, 0, 0, box, 0, 0, 0, box], np.float64)
    return systems.System(name="eam_pair", cell=cell, ltype=np.ones(n, np.int32), chge=np.zeros(n),
                          weight=np.full(n, 60.0), lfrzn=np.zeros(n, np.int32), vdw_prm=np.zeros(3),
                          x=np.array([-0.5 * r, 0.5 * r]), y=np.zeros(n), z=np.zeros(n), vx=np.zeros(n),
                          vy=np.zeros(n), vz=np.zeros(n), rcut=6.0, rpad=0.5, alpha=0.3, kmax=(16, 16, 16),
                          ntypes=ntypes, type_names=("M",))


def poly_tables(A=0.7, B=-0.3, C=0.05, a=2.0, b=-0.25, p=0.01, ng=400):
    """pair V = A + B r + C r^2, density rho = a + b r, embedding F = p rho^2 (all degree <= 2)."""
    r = np.linspace(1.0, 6.0, ng)
    rho = np.linspace(0.0, 10.0, ng)
    return [{"kind": "pair", "types": (1, 1), "start": 1.0, "finish": 6.0, "values": A + B * r + C * r * r},
            {"kind": "dens", "types": (1, 1), "start": 1.0, "finish": 6.0, "values": a + b * r},
            {"kind": "embe", "types": (1, 1), "start": 0.0, "finish": 10.0, "values": p * rho * rho}]


def kat_check(lib, r=2.7183, A=0.7, B=-0.3, C=0.05, a=2.0, b=-0.25, p=0.01):
    s = two_atoms(r)
    s.eam = poly_tables(A, B, C, a, b, p)
    lib.init(s)
    lib.start()
    e = lib.metal_energies()
    rho = a + b * r
    assert e["engmet"] == pytest.approx(A + B * r + C * r * r, rel=1e-12)
    assert e["engden"] == pytest.approx(2 * p * rho * rho, rel=1e-12)
    np.testing.assert_allclose(lib.metal_rho(), 2 * p * rho, rtol=1e-12)
    d = lib.download()
    # E(r) = V(r) + 2 F(rho(r)); atom 0 sits at -r/2: F_0 = +dE/dr along x
    dedr = (B + 2 * C * r) + 2 * (2 * p * rho) * b
    assert d["fx"][0] == pytest.approx(dedr, rel=1e-11)
    assert d["fx"][1] == pytest.approx(-dedr, rel=1e-11)
    assert abs(d["fy"][0]) < 1e-12 and abs(d["fz"][1]) < 1e-12
    assert e["virmet"] == pytest.approx(dedr * r, rel=1e-11)      # W = r dU/dr


def test_eam_known_answers_from_polynomial_tables(oracle_lib):
    for r in (1.3, 2.7183, 5.9):
        kat_check(oracle_lib, r=r)


def test_eam_forces_are_energy_gradients(oracle_lib):
    s = systems.eam_alloy(6)
    oracle_lib.init(s)
    oracle_lib.start()
    f = oracle_lib.download()
    assert np.abs(f["fx"].sum()) < 1e-8 * np.abs(f["fx"]).max() * s.natms

    def energy(dx, atom, comp):
        t = systems.eam_alloy(6)
        getattr(t, "xyz"[comp])[atom] += dx
        oracle_lib.init(t)
        oracle_lib.start()
        e = oracle_lib.metal_energies()
        return e["engmet"] + e["engden"]

    h = 1e-4
    for atom, comp in ((0, 0), (17, 1), (301, 2)):
        num = -(energy(h, atom, comp) - energy(-h, atom, comp)) / (2 * h)
        ana = f["xyz"[comp].replace("x", "fx").replace("y", "fy").replace("z", "fz")][atom]
        assert ana == pytest.approx(num, rel=2e-4, abs=1e-3 * np.abs(f["fx"]).std())


def test_eam_error_statuses(oracle_lib):
    s = two_atoms(0.9)                       # closer than the tables' first point
    s.eam = poly_tables()
    oracle_lib.init(s)
    with pytest.raises(Exception, match="506"):
        oracle_lib.start()
    s = two_atoms(2.0)
    tabs = poly_tables()
    tabs[2] = dict(tabs[2], start=5.0, finish=10.0)   # embedding starts above the local density
    s.eam = tabs
    oracle_lib.init(s)
    with pytest.raises(Exception, match="507"):
        oracle_lib.start()
