"""DL_POLY file formats on the host: CONFIG/REVCON, FIELD, CONTROL, STATIS, REVIVE.

Record layouts follow configuration.F90:2446 (write_config), ffield.F90 (FIELD
directives), control.F90:4501 (new-style CONTROL), statistics.F90:933 (STATIS) and
system.F90:1831 (REVIVE).  The runner test drives the host logic with the oracle
library as the path (CPU); the GPU run of the same files is in test_gpu_runner.py.
"""
import os
import struct

import numpy as np
import pytest

from dlpoly_gb300 import dlpoly_io as io
from dlpoly_gb300 import runner, systems


def test_fortran_edit_descriptors():
    assert io.fmt_g(1.5, 20, 10) == "     1.500000000    "
    assert io.fmt_g(-12.3456, 20, 10) == "    -12.34560000    "
    assert io.fmt_g(0.05, 20, 10) == "    0.5000000000E-01"
    assert io.fmt_g(0.1, 20, 10) == "    0.1000000000    "
    assert io.fmt_g(0.0, 20, 10) == "     0.000000000    "
    assert io.fmt_g(123456789012.0, 20, 10) == "    0.1234567890E+12"
    assert io.fmt_g(9.99999999999, 20, 10) == "     10.00000000    "   # rounds into the next decade
    assert io.fmt_e(0.002, 16, 7, 1) == "   2.0000000E-03"
    assert io.fmt_e(-1.5e-120, 14, 6, 1) == " -1.500000-120"
    assert io.fmt_e(0.0, 14, 6, 1) == "  0.000000E+00"
    assert io.fmt_e(12.5, 16, 10) == "0.1250000000E+02"
    assert io.fmt_f(45.12, 20, 10) == "       45.1200000000"
    assert io.fmt_i(12, 10) == "        12"
    assert io.fmt_i(10 ** 11, 10) == "*" * 10
    assert io.to_real("1.5D+02") == 150.0
    assert io.to_real("2.5-101") == 2.5e-101
    assert io.to_real("-.5E1") == -5.0


def _random_config(n, levcfg, imcon, seed=3):
    rng = np.random.default_rng(seed)
    cell = np.array([30.0, 0, 0, 2.5, 28.0, 0, -1.25, 3.0, 26.0]) if imcon == 3 else np.diag([30.0] * 3).ravel()
    pos = rng.uniform(-15, 15, (n, 3))
    pos[0] = [0.0, -1e-7, 1e7]                     # E-form and zero values
    return io.Config(title="random config", levcfg=levcfg, imcon=imcon, cell=cell,
                     names=["Na" if k % 3 else "Cl" for k in range(n)], index=np.arange(1, n + 1),
                     pos=pos, vel=rng.normal(0, 5, (n, 3)) if levcfg >= 1 else None,
                     frc=rng.normal(0, 3e3, (n, 3)) if levcfg >= 2 else None, step=17, tstep=0.001,
                     time=0.017)


@pytest.mark.parametrize("levcfg,imcon", [(0, 1), (1, 3), (2, 3), (2, 0)])
def test_config_round_trip(tmp_path, levcfg, imcon):
    c = _random_config(50, levcfg, imcon)
    p = tmp_path / "CONFIG"
    io.write_config(p, c)
    lines = p.read_text().split("\n")[:-1]
    assert all(len(x) == 72 for x in lines)                 # fixed 72-character records
    assert len(lines) == 2 + (3 if imcon else 0) + 50 * (levcfg + 2)
    r = io.read_config(p)
    assert (r.title, r.levcfg, r.imcon, r.step) == ("random config", levcfg, imcon, 17)
    assert r.tstep == pytest.approx(0.001) and r.time == pytest.approx(0.017)
    assert r.names == c.names and np.array_equal(r.index, c.index)
    if imcon:
        assert np.array_equal(r.cell, c.cell)
    for a, b in ((r.pos, c.pos), (r.vel, c.vel), (r.frc, c.frc)):
        if b is None:
            assert a is None
        else:                                               # g20.10: ten significant digits
            np.testing.assert_allclose(a, b, rtol=6e-10, atol=0)


def test_config_reader_orders_by_index(tmp_path):
    c = _random_config(20, 1, 1)
    perm = np.random.default_rng(0).permutation(20)
    shuffled = io.Config(title=c.title, levcfg=1, imcon=1, cell=c.cell, names=[c.names[k] for k in perm],
                         index=c.index[perm], pos=c.pos[perm], vel=c.vel[perm])
    io.write_config(tmp_path / "CONFIG", shuffled)
    r = io.read_config(tmp_path / "CONFIG")
    assert np.array_equal(r.index, np.arange(1, 21)) and r.names == c.names
    np.testing.assert_allclose(r.vel, c.vel, rtol=6e-10)


@pytest.mark.parametrize("make", [lambda: systems.nacl_melt(16), lambda: systems.spce_water(8)],
                         ids=["nacl_4096", "water_1536"])
def test_system_round_trip_through_files(tmp_path, make):
    s = make()
    perm = io.emit_inputs(s, tmp_path, steps=100, temperature=300.0, stats_every=10)
    assert sorted(perm.tolist()) == list(range(s.natms))
    ctl = io.read_control(tmp_path / "CONTROL")
    s2 = io.system_from_files(io.read_config(tmp_path / "CONFIG"), io.read_field(tmp_path / "FIELD"), ctl)
    assert s2.natms == s.natms and s2.ntypes == s.ntypes and s2.type_names == s.type_names
    assert np.array_equal(s2.ltype, s.ltype[perm])
    assert np.array_equal(s2.chge, s.chge[perm]) and np.array_equal(s2.weight, s.weight[perm])
    np.testing.assert_allclose(s2.vdw_prm, s.vdw_prm, rtol=1e-14)
    assert (s2.rcut, s2.rpad, s2.alpha, tuple(s2.kmax), s2.nsplines, s2.tstep, s2.shake_tol) == \
        (s.rcut, s.rpad, s.alpha, tuple(s.kmax), s.nsplines, s.tstep, s.shake_tol)
    for a, b in ((s2.x, s.x), (s2.y, s.y), (s2.vz, s.vz)):
        np.testing.assert_allclose(a, b[perm], rtol=6e-10, atol=1e-12)
    np.testing.assert_allclose(s2.cell, s.cell, rtol=0, atol=5.1e-11)   # f20.10 cell records
    assert s2.ntcons == s.ntcons
    if s.ntcons:                                            # water: molecules keep their order
        assert np.array_equal(perm, np.arange(s.natms))
        lc, lc2 = s.listcon.reshape(-1, 3), s2.listcon.reshape(-1, 3)
        assert np.array_equal(lc[:, 1:], lc2[:, 1:])
        assert np.array_equal(s.prmcon[lc[:, 0] - 1], s2.prmcon[lc2[:, 0] - 1])
        assert np.array_equal(s2.list_excl, s.list_excl)
    else:                                                   # NaCl: ions grouped by species
        assert np.all(np.diff(s2.ltype) >= 0)
    raw = np.load(tmp_path / "arrays.npz")
    assert np.array_equal(raw["x"], s.x) and np.array_equal(raw["perm"], perm)


def test_control_parser(tmp_path):
    p = tmp_path / "CONTROL"
    p.write_text("title  a test run  # comment\n"
                 "\n! whole-line comment\n"
                 "cutoff 1.2 nm\n"
                 "timestep 0.5 fs\n"
                 "time_run 250 steps\n"
                 "ensemble NVE\n"
                 "spme_kvec [24 &\n  30 36]\n"
                 "spme_alpha 0.03 nm^-1\n"
                 "shake_tolerance 1.0d-8 ang\n"
                 "spme_nsplines 7\n")
    c = io.read_control(p)
    assert c["title"] == "a test run"
    assert c["cutoff"] == pytest.approx(12.0) and c["timestep"] == pytest.approx(5e-4)
    assert c["time_run"] == 250 and c["ensemble"] == "nve"
    assert c["spme_kvec"] == [24, 30, 36] and c["spme_alpha"] == pytest.approx(0.003)
    assert c["shake_tolerance"] == 1e-8
    s = io.system_from_files(_random_config(2, 0, 1), io.Field("f", "kj", [
        io.MoleculeType("Cl", 1, [io.Site("Cl", 35.45, -1.0)]),
        io.MoleculeType("Na", 1, [io.Site("Na", 22.99, 1.0)])], []),
        dict(c, coul_method="spme"))
    assert s.nsplines == 8                                  # odd orders round up (control.F90:1665)
    for text, msg in (("title t\nbogus_key 1\n", "Unrecognised key"),
                      ("title t\ncutoff 1 ang\ncutoff 2 ang\n", "already set"),
                      ("cutoff 10\n", "old-style"),
                      ("title t\nspme_nsplines 8 9\n", "junk"),
                      ("title t\ncutoff 10 furlong\n", "unit")):
        p.write_text(text)
        with pytest.raises(ValueError, match=msg):
            io.read_control(p)


def test_gbcontrol_keys(tmp_path):
    io.write_control(tmp_path / "GBCONTROL", {"gb_precision": "mixed", "gb_mts_k": 4, "gb_mts_tol": 1e-4},
                     io.GB_KEYS)
    g = io.read_control(tmp_path / "GBCONTROL", io.GB_KEYS)
    assert g == {"gb_precision": "mixed", "gb_mts_k": 4, "gb_mts_tol": 1e-4}


def test_spme_parameters_from_precision():
    """control.F90:1705-1711 for 'spme_precision 1e-6': the alpha and grid sizes the
    reference derives for the NaCl boxes (rc 12 A) and the water box (rc 10 A)."""
    for rc, L, alpha, k in ((12.0, 45.12, 0.26506, 24), (12.0, 180.48, 0.26506, 98), (10.0, 99.3, 0.32080, 64)):
        a, kv = io.spme_kvec_from_precision(1e-6, rc, np.diag([L] * 3).ravel())
        assert a == pytest.approx(alpha, abs=5e-6) and kv == (k, k, k)


def test_field_reader_directives(tmp_path):
    p = tmp_path / "FIELD"
    p.write_text("ions in eV\nunits eV\nmolecules 1\nsalt pair\nnummols 3\natoms 4\n"
                 "  Na 22.99 1.0 2 1\n Cl 35.45 -1.0\n# a comment\nCl 35.45 -1.0 1 0\n"
                 "bonds 0\nfinish\nvdw 1\nNa Cl lj 0.01 3.0\nclose\n")
    f = io.read_field(p)
    m = f.molecules[0]
    assert (f.units, m.name, m.nummols, len(m.sites)) == ("ev", "salt pair", 3, 4)
    assert [x.freeze for x in m.sites] == [1, 1, 0, 0] and f.unique_names() == ["Na", "Cl"]
    assert f.vdw == [("Na", "Cl", "lj", (0.01, 3.0))]
    cfg = io.Config("c", 0, 1, np.diag([20.0] * 3).ravel(), ["Na", "Na", "Cl", "Cl"] * 3, np.arange(1, 13),
                    np.random.default_rng(1).uniform(-9, 9, (12, 3)))
    s = io.system_from_files(cfg, f, {"cutoff": 8.0, "coul_method": "spme", "spme_alpha": 0.3,
                                      "spme_kvec": [16, 16, 16]})
    assert s.vdw_prm[3:6].tolist() == [1.0, 0.01 * 9648.530821, 3.0]     # key (2,1), eV -> internal
    assert s.lfrzn.tolist() == [1, 1, 0, 0] * 3
    for body, exc in (("bonds 1\n1 2 harm 1.0 1.0\n", NotImplementedError),
                      ("shell 1 1\n1 2 10.0\n", NotImplementedError)):
        p.write_text("t\nunits kj\nmolecules 1\nm\nnummols 1\natoms 2\nA 1.0 0.0 2\n" + body + "finish\nclose\n")
        with pytest.raises(exc):
            io.read_field(p)
    p.write_text("t\nunits kj\nmolecules 1\nm\nnummols 1\natoms 1\nA 1.0 0.0\nfinish\nvdw 1\nA A buck 1 1 1\nclose\n")
    with pytest.raises(NotImplementedError):
        io.read_field(p)
    cfg.names[0] = "Cl"
    with pytest.raises(ValueError, match="CONFIG atom 1"):
        io.system_from_files(cfg, f, {"cutoff": 8.0, "coul_method": "spme", "spme_alpha": 0.3,
                                      "spme_kvec": [16, 16, 16]})


def test_vdw_long_range_matches_quadrature():
    from scipy.integrate import quad

    s = systems.nacl_melt(16)
    elrc, vlrc = io.vdw_long_range(s)
    vol = s.volume()
    num = np.bincount(s.ltype)[1:]
    e = v = 0.0
    for a in (1, 2):
        for b in (1, 2):
            hi, lo = max(a, b), min(a, b)
            k = hi * (hi - 1) // 2 + lo - 1
            eps, sig = s.vdw_prm[3 * k + 1], s.vdw_prm[3 * k + 2]
            u = lambda r: 4 * eps * ((sig / r) ** 12 - (sig / r) ** 6)
            du = lambda r: 4 * eps * (-12 * sig ** 12 / r ** 13 + 6 * sig ** 6 / r ** 7)
            e += 2 * np.pi / vol * num[a - 1] * num[b - 1] * quad(lambda r: r * r * u(r), s.rcut, np.inf)[0]
            v += 2 * np.pi / vol * num[a - 1] * num[b - 1] * quad(lambda r: r ** 3 * du(r), s.rcut, np.inf)[0]
    assert elrc == pytest.approx(e, rel=1e-9) and vlrc == pytest.approx(v, rel=1e-9)


def test_statistics_accumulators_and_records(tmp_path):
    s = systems.nacl_melt(16)
    st = io.Statistics(s, units="kj")
    assert st.mxnstk == 53 and st.mxstak == 100 and st.degfre == 3 * s.natms - 3
    rng = np.random.default_rng(5)
    hist = []
    for n in range(0, 151):
        d = {k: rng.normal() * 1e3 for k in ("engcpe_rc", "vircpe_rc", "engcpe_rl", "vircpe_rl", "engcpe_ex",
                                             "vircpe_ex", "engvdw", "virvdw", "vircon")}
        d["engke"] = 1e4 + rng.normal()
        d["stress"], d["strkin"], d["strcon"] = rng.normal(size=9), rng.normal(size=9), rng.normal(size=9)
        st.collect(n, d, s.cell, amsd=[1.0 * n, 2.0 * n])
        if n:
            hist.append(st.stpval.copy())
    h = np.array(hist)
    assert st.numacc == 150
    np.testing.assert_allclose(st.sumval, (h - h[0]).mean(0), rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(st.ssqval, (h - h[0]).var(0), rtol=1e-8, atol=1e-9)
    np.testing.assert_allclose(st.ravval, h[-100:].mean(0), rtol=1e-9, atol=1e-9)
    v = st.stpval
    assert v[1] == pytest.approx(v[3] + d["engke"] / 100.0)                 # total = cfg + kinetic
    assert v[2] == pytest.approx(2 * d["engke"] / (io.BOLTZ * st.degfre))   # temperature
    assert v[37] == pytest.approx(150.0 / 2048) and v[38] == pytest.approx(300.0 / 2048)
    rec = st.statis_record(150, 0.3).split("\n")[:-1]
    assert rec[0] == "       150  3.000000E-01        39"
    assert len(rec) == 1 + 8 and all(len(x) == 70 for x in rec[1:-1]) and len(rec[-1]) == 56
    assert float(rec[1].split()[0]) == pytest.approx(v[1], rel=1e-6)
    assert st.header("t") == "title: 't'\nenergy unitS: kjoule/mol\n"
    st.write_revive(tmp_path / "REVIVE", s.rcut, s.natms, 150, 0.002, 0.3, 0.0, d["strcon"], d["stress"])
    raw = (tmp_path / "REVIVE").read_bytes()
    assert struct.unpack_from("<i", raw, 0)[0] == 24 and struct.unpack_from("<i", raw, 28)[0] == 24
    st2 = io.Statistics(s, units="kj")
    info = st2.read_revive(tmp_path / "REVIVE")
    assert info["nstep"] == 150 and info["megatm"] == s.natms and st2.numacc == 150
    for name in ("stpval", "sumval", "ssqval", "zumval", "ravval", "stkval", "stpvl0"):
        assert np.array_equal(getattr(st2, name), getattr(st, name)), name


def test_runner_host_logic_on_oracle(tmp_path, oracle_lib):
    """Emit -> run -> STATIS / REVCON / REVIVE -> continue, driven through the oracle
    library on the CPU (the GPU run of the same files is a gpu test)."""
    d = str(tmp_path)
    runner.emit("water_1536", d, steps=10, stats_every=5)
    with open(os.path.join(d, "CONTROL"), "a") as fh:
        fh.write("data_dump_frequency 5 steps\n")
    out = runner.run(d, lib=oracle_lib, quiet=True)
    assert out["final_step"] == 10
    statis = open(os.path.join(d, "STATIS")).read().split("\n")
    heads = [x for x in statis if len(x) == 34]
    assert [int(x[:10]) for x in heads] == [0, 5, 10] and all(int(x[24:]) == 39 for x in heads)
    rev = io.read_config(os.path.join(d, "REVCON"))
    assert (rev.levcfg, rev.step) == (2, 10) and rev.time == pytest.approx(0.02)
    fin = oracle_lib.download()
    np.testing.assert_allclose(rev.pos[:, 0], fin["x"], rtol=6e-10, atol=1e-12)
    np.testing.assert_allclose(rev.frc[:, 2], fin["fz"], rtol=6e-10, atol=1e-9)
    # the same files run directly through the path give the STATIS energies
    cfg = io.read_config(os.path.join(d, "CONFIG"))
    s = io.system_from_files(cfg, io.read_field(os.path.join(d, "FIELD")), io.read_control(os.path.join(d, "CONTROL")))
    oracle_lib.init(s)
    oracle_lib.start()
    last = oracle_lib.md_vv(10)[-1]
    elrc, _ = io.vdw_long_range(s)
    tot = (last.engcpe_rc + last.engcpe_rl + last.engcpe_ex + last.engvdw + elrc + last.engke) / 100.0
    assert float(statis[statis.index(heads[-1]) + 1].split()[0]) == pytest.approx(tot, rel=1e-6)
    # continue from REVCON/REVIVE for 5 more steps: STATIS appended, steps count on
    os.replace(os.path.join(d, "REVCON"), os.path.join(d, "CONFIG"))
    txt = open(os.path.join(d, "CONTROL")).read().replace("restart noscale", "restart continue")
    txt = txt.replace("time_run 10 steps", "time_run 5 steps")
    open(os.path.join(d, "CONTROL"), "w").write(txt)
    out = runner.run(d, lib=oracle_lib, quiet=True)
    assert out["final_step"] == 15
    heads = [x for x in open(os.path.join(d, "STATIS")).read().split("\n") if len(x) == 34]
    assert [int(x[:10]) for x in heads] == [0, 5, 10, 15]
    assert io.read_config(os.path.join(d, "REVCON")).step == 15


def test_ensemble_keys_of_control(tmp_path):
    p = tmp_path / "CONTROL"
    p.write_text("title t\nensemble nvt\nensemble_method Hoover\nensemble_thermostat_coupling 50 fs\n"
                 "temperature 300 K\nrandom_seed [1 2 3]\n")
    e = io.ensemble_from_control(io.read_control(p))
    assert e == {"kind": "nose-hoover", "temp": 300.0, "tau_t": pytest.approx(0.05), "chi": 0.0, "seed": (1, 2, 3)}
    p.write_text("title t\nensemble nvt\nensemble_method langevin\nensemble_thermostat_friction 2 ps^-1\n"
                 "temperature 300 K\n")
    assert io.ensemble_from_control(io.read_control(p))["chi"] == 2.0
    for bad in ("ensemble npt\n", "ensemble nvt\nensemble_method andersen\n"):
        p.write_text("title t\n" + bad)
        with pytest.raises(NotImplementedError):
            io.ensemble_from_control(io.read_control(p))


def test_runner_nose_hoover_restart_on_oracle(tmp_path, oracle_lib):
    """NVT Nose-Hoover from CONTROL: STATIS carries the conserved-energy term and a
    continued run restores chi_t and cint from REVIVE."""
    d = str(tmp_path)
    runner.emit("nacl_4096", d, steps=6, stats_every=3)
    ctl = os.path.join(d, "CONTROL")
    txt = open(ctl).read().replace("ensemble nve", "ensemble nvt\nensemble_method hoover\n"
                                   "ensemble_thermostat_coupling 0.05 ps")
    open(ctl, "w").write(txt)
    runner.run(d, lib=oracle_lib, quiet=True)
    th = oracle_lib.thermostat_state()
    assert th["consv"] != 0.0
    s = io.system_from_files(io.read_config(os.path.join(d, "REVCON")), io.read_field(os.path.join(d, "FIELD")),
                             io.read_control(ctl))
    info = io.Statistics(s).read_revive(os.path.join(d, "REVIVE"))
    assert (info["chi_t"], info["cint"]) == (th["chi_t"], th["cint"])
    rec = [x for x in open(os.path.join(d, "STATIS")).read().split("\n") if x]
    last = rec[rec.index([x for x in rec if len(x) == 34][-1]) + 6].split()
    assert float(last[2]) == pytest.approx(th["consv"] / 100.0, rel=1e-6)    # stpval(0) follows stpval(1:27)
    os.replace(os.path.join(d, "REVCON"), os.path.join(d, "CONFIG"))
    txt = open(ctl).read().replace("restart noscale", "restart continue").replace("time_run 6 steps", "time_run 3 steps")
    open(ctl, "w").write(txt)
    out = runner.run(d, lib=oracle_lib, quiet=True)
    assert out["final_step"] == 9
    assert oracle_lib.thermostat_state()["cint"] != th["cint"]


def test_eam_inputs_round_trip(tmp_path, oracle_lib):
    """FIELD 'metal ... eam' + TABEAM written and read back give the same system: the
    oracle's metal energies agree (atoms are regrouped by species, types renumbered)."""
    s = systems.eam_alloy(6)
    io.emit_inputs(s, tmp_path, steps=10, temperature=600.0)
    fld = io.read_field(tmp_path / "FIELD")
    assert fld.units == "ev" and sorted(fld.metal) == sorted([("Cu", "Cu", "eam"), ("Ni", "Cu", "eam"),
                                                               ("Ni", "Ni", "eam")])
    ctl = io.read_control(tmp_path / "CONTROL")
    assert ctl["coul_method"] == "off"
    s2 = io.system_from_files(io.read_config(tmp_path / "CONFIG"), fld, ctl, tabeam=str(tmp_path / "TABEAM"))
    assert len(s2.eam) == 7 and s2.metal_listed.tolist() == [1, 1, 1]
    t_in = {(t["kind"], tuple(s.type_names[k - 1] for k in t["types"])): t for t in s.eam}
    for t in s2.eam:
        u = t_in[(t["kind"], tuple(s2.type_names[k - 1] for k in t["types"]))]
        np.testing.assert_allclose(t["values"], u["values"], rtol=1e-15, atol=0)
        assert (t["start"], t["finish"]) == (u["start"], u["finish"])
    energies = []
    for sys_ in (s, s2):
        oracle_lib.init(sys_)
        oracle_lib.start()
        e = oracle_lib.metal_energies()
        energies.append(e["engmet"] + e["engden"])
    assert energies[1] == pytest.approx(energies[0], rel=1e-9)
    bad = tmp_path / "FIELD2"
    bad.write_text(open(tmp_path / "FIELD").read().replace("Cu       Cu       eam", "Cu       Cu       fnsc 1 2 3 4 5"))
    with pytest.raises(NotImplementedError):
        io.read_field(bad)
