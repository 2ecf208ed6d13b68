"""GPU parity: the CUDA path against the FP64 oracle on the same seeded inputs,
through the C-ABI (gb_* entry points).

Bars: pair sets bit-exact; FP64 forces within 1e-10 of
the oracle (max |dF| relative to the rms force); energies and virials within
1e-10 relative; mixed form rms force error <= 1e-5 relative.
"""
import numpy as np
import pytest

from conftest import force_dev, force_rms_rel
from dlpoly_gb300 import systems

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10
CASES = {
    "nacl_4096": lambda: systems.nacl_melt(16),
    "water_1536": lambda: systems.spce_water(8),
    "water_5184": lambda: systems.spce_water(12),
    "nacl_13824": lambda: systems.nacl_melt(24, kmax=72),
}


def _pair(gpu_lib, oracle_lib, s, precision=0, **kw):
    gpu_lib.init(s, precision=precision, **kw)
    oracle_lib.init(s, **kw)
    gpu_lib.relocate()
    oracle_lib.relocate()


@pytest.mark.parametrize("name", list(CASES))
def test_pair_set_bit_exact(gpu_lib, oracle_lib, name):
    s = CASES[name]()
    _pair(gpu_lib, oracle_lib, s)
    ld = gpu_lib.link_cell_pairs()
    lr = oracle_lib.link_cell_pairs()
    # the whole list(-3:max_list, natms) array: markers, entries and their order
    assert np.array_equal(ld, lr)


@pytest.mark.parametrize("precision", [0, 2], ids=["fp64", "fp64_native"])
@pytest.mark.parametrize("name", list(CASES))
def test_forces_fp64(gpu_lib, oracle_lib, name, precision):
    """The FP64 form (pair loop in double-float) and its all-native-FP64 variant."""
    s = CASES[name]()
    _pair(gpu_lib, oracle_lib, s, precision=precision)
    gpu_lib.link_cell_pairs(want_list=False)
    oracle_lib.link_cell_pairs(want_list=False)
    ed, sd = gpu_lib.two_body_forces()
    er, sr = oracle_lib.two_body_forces()
    assert force_dev(gpu_lib.download(), oracle_lib.download()) < FP64_TOL
    for k in er:
        assert abs(ed[k] - er[k]) <= FP64_TOL * max(abs(er[k]), 1.0), (k, ed[k], er[k])
    assert np.abs(sd - sr).max() <= FP64_TOL * np.abs(sr).max()


def test_spme_alone_fp64(gpu_lib, oracle_lib):
    s = systems.nacl_melt(16)
    _pair(gpu_lib, oracle_lib, s)
    ed, vd, sd = gpu_lib.ewald_spme_forces()
    er, vr, sr = oracle_lib.ewald_spme_forces()
    assert ed == pytest.approx(er, rel=FP64_TOL)
    assert vd == pytest.approx(vr, rel=1e-9)
    assert force_dev(gpu_lib.download(), oracle_lib.download()) < FP64_TOL


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_spme_with_uncharged_atoms(gpu_lib, oracle_lib, precision):
    """Atoms without charge take no part in the spread (no brick) and gather nothing: their
    reciprocal force is only the removal of the mean net force, the same for each of them,
    and every atom's force matches the oracle (FP64 bar, or the mixed form's error bound)."""
    s = systems.nacl_melt(16)
    q = s.chge.copy()
    q[np.flatnonzero(q > 0)[::7]] = 0.0
    q[np.flatnonzero(q < 0)[::7]] = 0.0
    s.chge = q
    _pair(gpu_lib, oracle_lib, s, precision=precision)
    ed, vd, sd = gpu_lib.ewald_spme_forces()
    er, vr, sr = oracle_lib.ewald_spme_forces()
    a, b = gpu_lib.download(), oracle_lib.download()
    z = q == 0.0
    for k in ("fx", "fy", "fz"):
        assert np.ptp(a[k][z]) == 0.0, k
    if precision == 0:
        assert ed == pytest.approx(er, rel=FP64_TOL)
        assert force_dev(a, b) < FP64_TOL
    else:  # FP32 grid arithmetic, relative to the reciprocal force alone
        assert ed == pytest.approx(er, rel=1e-5)
        assert force_rms_rel(a, b) <= 1e-4


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("order", [4, 6, 10, 12])
def test_spme_spline_orders(gpu_lib, oracle_lib, order, precision):
    """Spline orders other than the workloads' 8: order 6 through the kernels instantiated
    for it (the warp gathers included), 4, 10 and 12 through the run-time-order kernels
    (the spread's plane-per-warp branch above order 8 among them)."""
    s = systems.nacl_melt(16)
    s.nsplines = order
    _pair(gpu_lib, oracle_lib, s, precision=precision)
    ed, vd, sd = gpu_lib.ewald_spme_forces()
    er, vr, sr = oracle_lib.ewald_spme_forces()
    a, b = gpu_lib.download(), oracle_lib.download()
    if precision == 0:
        assert ed == pytest.approx(er, rel=FP64_TOL)
        assert vd == pytest.approx(vr, rel=1e-9)
        assert force_dev(a, b) < FP64_TOL
    else:
        assert ed == pytest.approx(er, rel=1e-5)
        assert force_rms_rel(a, b) <= 1e-4


def test_md_atoms_below_lower_face(gpu_lib, oracle_lib):
    """Between relocations an atom can drift below the cell's lower face, where its
    fractional grid coordinate u is negative: the spread takes floor(u) and u - floor(u),
    the gather Int(u) and u - Aint(u) (ewald_spole.F90:387), so the two use different
    splines for that atom.  The NaCl lattice shifted by -1.35 A puts a layer of atoms at
    the lower faces; 8 steps without a list rebuild carry dozens of them across (the
    oracle's halo images stand in for them in its spread), against the oracle."""
    s = systems.nacl_melt(16)
    L = s.cell[0]
    for c in ("x", "y", "z"):
        setattr(s, c, getattr(s, c) - 1.35)
    gpu_lib.init(s)
    oracle_lib.init(s)
    gpu_lib.start()
    oracle_lib.start()
    sd = gpu_lib.md_vv(8)
    sr = oracle_lib.md_vv(8)
    assert [x.list_rebuilt for x in sd] == [x.list_rebuilt for x in sr]
    assert not any(x.list_rebuilt for x in sr)
    a, b = gpu_lib.download(), oracle_lib.download()
    assert sum(int((b[c] < -0.5 * L).sum()) for c in ("x", "y", "z")) >= 20
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.abs(a[k] - b[k]).max() <= 1e-9 * np.abs(b[k]).max(), k
    assert force_dev(a, b) < 1e-8
    for x, y in zip(sd, sr):
        assert x.engcpe_rc == pytest.approx(y.engcpe_rc, rel=1e-9)
        assert x.engcpe_rl == pytest.approx(y.engcpe_rl, rel=1e-9)


def test_vdw_known_answer_on_gpu(gpu_lib):
    """source/unit_tests/test_vdw.F90:46-59 entry 2 (LJ eps=1 sigma=2 at r=1) through the device path."""
    s = systems.lj_pair(eps=1.0, sigma=2.0, r=1.0)
    gpu_lib.init(s)
    gpu_lib.relocate()
    gpu_lib.link_cell_pairs(want_list=False)
    e, _ = gpu_lib.real_space_forces()
    assert e["engvdw"] == pytest.approx(16128.0, rel=1e-13)
    assert e["virvdw"] == pytest.approx(-195072.0, rel=1e-13)
    d = gpu_lib.download()
    assert d["fx"][1] == pytest.approx(195072.0, rel=1e-13)


@pytest.mark.parametrize("name,nsteps", [("nacl_4096", 30), ("water_1536", 12)])
def test_md_steps_fp64(gpu_lib, oracle_lib, name, nsteps):
    """Resident md_vv loop (VV + SHAKE/RATTLE + conditional list rebuild) step by step."""
    s = CASES[name]()
    gpu_lib.init(s)
    oracle_lib.init(s)
    gpu_lib.start()
    oracle_lib.start()
    sd = gpu_lib.md_vv(nsteps)
    sr = oracle_lib.md_vv(nsteps)
    assert [x.list_rebuilt for x in sd] == [x.list_rebuilt for x in sr]
    assert any(x.list_rebuilt for x in sr) or name.startswith("water")
    assert [x.shake_iters for x in sd] == [x.shake_iters for x in sr]
    assert [x.rattle_iters for x in sd] == [x.rattle_iters for x in sr]
    a, b = gpu_lib.download(), oracle_lib.download()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        scale = np.abs(b[k]).max()
        assert np.abs(a[k] - b[k]).max() <= 1e-9 * scale, k
    assert force_dev(a, b) < 1e-8
    for x, y in zip(sd, sr):
        assert x.engke == pytest.approx(y.engke, rel=1e-9)
        assert x.engcpe_rl == pytest.approx(y.engcpe_rl, rel=1e-9)
        cs = max(np.abs(y.strcon[:]).max(), 1e-30)
        assert np.abs(np.array(x.strcon[:]) - np.array(y.strcon[:])).max() <= 1e-8 * cs


def test_cluster_constraints_match_global_sweeps(gpu_lib, monkeypatch):
    """Cluster-local SHAKE/RATTLE (one thread per rigid molecule, one grid
    barrier per chunk of sweeps) against the per-sweep global kernels: same
    iteration counts and the same trajectory."""
    s = systems.spce_water(12)
    runs = []
    # per-sweep global kernels, then one thread per cluster
    for glob in ("1", "0"):
        monkeypatch.setenv("GB_SHAKE_GLOBAL", glob)
        gpu_lib.init(s)
        gpu_lib.start()
        st = gpu_lib.md_vv(20)
        runs.append((st, gpu_lib.download()))
    sg, a = runs[0]
    assert max(x.shake_iters for x in sg) > 1
    for sc, b in runs[1:]:
        assert [x.shake_iters for x in sg] == [x.shake_iters for x in sc]
        assert [x.rattle_iters for x in sg] == [x.rattle_iters for x in sc]
        # same update arithmetic; last-bit differences from FMA contraction grow
        # through 20 chaotic steps to ~1e-12 relative, the oracle comparison's bar is 1e-9
        for k in ("x", "y", "z", "vx", "vy", "vz"):
            assert np.abs(a[k] - b[k]).max() <= 1e-9 * np.abs(a[k]).max(), k
        for x, y in zip(sg, sc):
            assert x.vircon == pytest.approx(y.vircon, rel=1e-8, abs=1e-6)


def test_md_matches_golden(gpu_lib):
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "nacl_4096.npz"))
    s = systems.nacl_melt(16)
    gpu_lib.init(s)
    gpu_lib.relocate()
    lst = gpu_lib.link_cell_pairs()
    assert np.array_equal(lst[:, 3], g["list_count"])
    gpu_lib.two_body_forces()
    d = gpu_lib.download()
    F = np.stack([d["fx"], d["fy"], d["fz"]], 1)
    assert np.abs(F - g["f0"]).max() / np.sqrt((g["f0"] ** 2).sum(1).mean()) < FP64_TOL
    gpu_lib.md_vv(5)
    d = gpu_lib.download()
    assert np.abs(np.stack([d["x"], d["y"], d["z"]], 1) - g["x5"]).max() < 1e-9


@pytest.mark.parametrize("name", ["nacl_4096", "water_5184"])
def test_mixed_force_error(gpu_lib, oracle_lib, name):
    s = CASES[name]()
    _pair(gpu_lib, oracle_lib, s, precision=1)
    gpu_lib.link_cell_pairs(want_list=False)
    oracle_lib.link_cell_pairs(want_list=False)
    ed, _ = gpu_lib.two_body_forces()
    er, _ = oracle_lib.two_body_forces()
    a, b = gpu_lib.download(), oracle_lib.download()
    assert force_rms_rel(a, b) <= 1e-5
    keys = ("engcpe_rc", "engcpe_rl", "engcpe_ex", "engvdw")
    tot_d = sum(ed[k] for k in keys)
    tot_r = sum(er[k] for k in keys)
    # FP32 pair/grid energies: error bounded by the magnitude of the terms,
    # which cancel heavily for water (reciprocal vs exclusion correction)
    assert abs(tot_d - tot_r) <= 2e-6 * sum(abs(er[k]) for k in keys)
    assert ed["engcpe_ex"] == pytest.approx(er["engcpe_ex"], rel=1e-10)  # FP64 in both forms


def test_mixed_is_deterministic(gpu_lib):
    """Fixed-point force sums: two runs give bit-identical forces and trajectories."""
    out = []
    for _ in range(2):
        gpu_lib.init(systems.nacl_melt(16), precision=1)
        gpu_lib.start()
        gpu_lib.md_vv(10)
        out.append(gpu_lib.download())
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


def test_list_overflow_status(gpu_lib):
    s = systems.nacl_melt(16)
    gpu_lib.init(s, max_list=50)
    gpu_lib.relocate()
    st, need = gpu_lib.list_build_status()
    assert st == 106 and need > 50
    # the context stays usable: a later call with a fresh init works
    gpu_lib.init(s)
    gpu_lib.relocate()
    assert gpu_lib.list_build_status()[0] == 0


def test_nonfinite_positions_rejected(gpu_lib):
    s = systems.nacl_melt(16)
    gpu_lib.init(s)
    x = s.x.copy()
    x[7] = np.nan
    with pytest.raises(Exception) as e:
        gpu_lib.upload(x, s.y, s.z)
    assert getattr(e.value, "code", None) == -5


def test_cutoff_larger_than_half_cell_rejected(gpu_lib):
    s = systems.nacl_melt(16)
    s.rcut = 22.0
    with pytest.raises(Exception) as e:
        gpu_lib.init(s)
    assert getattr(e.value, "code", None) == 95


def test_shake_nonconvergence_status(gpu_lib):
    """SHAKE that does not converge within shake_maxit returns 105 (constraints.F90:996);
    the context stays usable for a clean run afterwards."""
    s = systems.spce_water(8)
    gpu_lib.init(s, shake_maxit=2)  # the lattice start needs ~65 sweeps at tolerance 1e-8
    gpu_lib.start()
    with pytest.raises(Exception) as e:
        gpu_lib.md_vv(1)
    assert getattr(e.value, "code", None) == 105
    gpu_lib.init(s)
    gpu_lib.start()
    st = gpu_lib.md_vv(2)
    assert all(x.shake_iters > 2 for x in st)


def test_rattle_nonconvergence_status(gpu_lib):
    """RATTLE that does not converge within shake_maxit returns 515 (constraints.F90:748)."""
    s = systems.spce_water(8)
    gpu_lib.init(s, shake_maxit=2)
    gpu_lib.start()
    d = gpu_lib.download()
    rng = np.random.default_rng(7)
    # velocities far off the constraint manifold: RATTLE needs many sweeps
    v = [d[k] + rng.normal(0.0, 5.0, s.natms) for k in ("vx", "vy", "vz")]
    gpu_lib.upload(d["x"], d["y"], d["z"], *v)
    gpu_lib.constraints_tags()
    with pytest.raises(Exception) as e:
        gpu_lib.apply_rattle()
    assert getattr(e.value, "code", None) == 515
    gpu_lib.init(s)
    gpu_lib.start()
    assert all(x.rattle_iters > 2 for x in gpu_lib.md_vv(2))


def test_halo_overflow_status(gpu_lib):
    """More halo images than mxatms holds returns 56 (deport_data.F90:1870)."""
    s = systems.nacl_melt(16)
    gpu_lib.init(s, mxatms=s.natms + 64)
    with pytest.raises(Exception) as e:
        gpu_lib.relocate()
    assert getattr(e.value, "code", None) == 56
    gpu_lib.init(s)
    gpu_lib.relocate()
    assert gpu_lib.list_build_status()[0] == 0


def test_multi_rank_rejected(gpu_lib):
    """A run with more than one MPI rank (comm%mxnode > 1) cannot use the device path."""
    s = systems.nacl_melt(16)
    with pytest.raises(Exception) as e:
        gpu_lib.init(s, mxnode=2)
    assert getattr(e.value, "code", None) == -8
    gpu_lib.init(s, mxnode=1)


def test_mts_rejects_cutoff_below_descriptor_reach(gpu_lib):
    """The learned form's neighbour sums reach 6 A: a shorter pair cutoff is refused."""
    s = systems.nacl_melt(16, rcut=5.0)
    gpu_lib.init(s, precision=1)
    with pytest.raises(Exception) as e:
        gpu_lib.mts_config(4, 1e-4, 10)
    assert getattr(e.value, "code", None) == -3


def test_shake_rattle_exports_match_vv(gpu_lib):
    """gb_constraints_tags + a host-side stage update + gb_shake / gb_rattle (the
    apply_shake / apply_rattle shims) give the same state as gb_vv's stages."""
    s = systems.spce_water(8)
    out = []
    for split in (False, True):
        gpu_lib.init(s)
        gpu_lib.start()
        dt = s.tstep
        if not split:
            a = gpu_lib.nve_0_vv(1)
            gpu_lib.refresh()
            gpu_lib.two_body_forces()
            b_it = gpu_lib.nve_0_vv(2)["iters"]
            out.append((gpu_lib.download(), a["iters"], b_it, a["strcon"]))
            continue
        d = gpu_lib.download()
        gpu_lib.constraints_tags()
        m = s.weight
        v = [d[k] + 0.5 * dt / m * d[f] for k, f in (("vx", "fx"), ("vy", "fy"), ("vz", "fz"))]
        x = [d[k] + dt * vv for k, vv in zip(("x", "y", "z"), v)]
        gpu_lib.upload(*x, *v)
        sh = gpu_lib.apply_shake()
        gpu_lib.refresh()
        gpu_lib.two_body_forces()
        d = gpu_lib.download()
        gpu_lib.constraints_tags()
        v = [d[k] + 0.5 * dt / m * d[f] for k, f in (("vx", "fx"), ("vy", "fy"), ("vz", "fz"))]
        gpu_lib.upload(d["x"], d["y"], d["z"], *v)
        r_it = gpu_lib.apply_rattle()
        out.append((gpu_lib.download(), sh["iters"], r_it, sh["strcon"]))
    (a, sa, ra, ca), (b, sb, rb, cb) = out
    assert (sa, ra) == (sb, rb) and sa > 1 and ra > 1
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.abs(a[k] - b[k]).max() <= 1e-12 * np.abs(a[k]).max(), k
    assert np.abs(ca - cb).max() <= 1e-10 * np.abs(ca).max()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name", ["nacl_4096", "water_5184"])
def test_sorted_pair_kernels_match_atom_index_kernels(gpu_lib, monkeypatch, name, precision):
    """The pair kernels over the sorted-position list (partners in cell order, halo pairs
    from their forward copy) against the atom-index kernels on the same list: forces and
    energies agree to rounding and every forward halo entry has its backward copy.  A small
    first-launch capacity of the tiled list build (most tiles in its second launch) changes
    nothing."""
    s = CASES[name]()
    runs = {}
    for mode, env in (("atom", {"GB_PAIR_SORTED": "0"}), ("sorted", {}), ("small_cap", {"GB_TILE_CAP": "64"})):
        monkeypatch.delenv("GB_PAIR_SORTED", raising=False)
        monkeypatch.delenv("GB_TILE_CAP", raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        gpu_lib.init(s, precision=precision)
        gpu_lib.relocate()
        lst = gpu_lib.link_cell_pairs()
        e, st = gpu_lib.two_body_forces()
        runs[mode] = (e, st, gpu_lib.download(), gpu_lib.pair_counts(), lst)
    monkeypatch.delenv("GB_TILE_CAP", raising=False)
    a = runs["atom"]
    for mode in ("sorted", "small_cap"):
        b = runs[mode]
        cnt = b[3]
        assert cnt[5] == 1, mode  # the sorted-position kernels ran
        assert cnt[3] == cnt[4] and cnt[3] > 0
        assert cnt[0] == a[3][0] and cnt[1] == a[3][1]  # same list entries and pairs inside rc
        assert np.array_equal(b[4], a[4])
        # the two kernels evaluate a halo pair from opposite sides: double-float rounding (~1e-12)
        tol = 1e-11 if precision == 0 else 1e-5
        assert force_dev(b[2], a[2]) < tol, mode
        for k in a[0]:
            assert abs(b[0][k] - a[0][k]) <= tol * max(abs(a[0][k]), 1.0), (mode, k)
        assert np.abs(b[1] - a[1]).max() <= tol * np.abs(a[1]).max()
    assert runs["small_cap"][3][6] > 0  # the list build's second launch ran


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_pair_kernel_cta_sizes_agree(gpu_lib, monkeypatch, precision):
    """The sorted pair kernels in one resident set of 1024-thread CTAs (the FP64 form's
    default), in 256-thread CTAs, and in short-lived CTAs of 16 atoms per warp (the mixed
    form's default) hand the atoms to warps in other orders: the fixed-point forces are
    bit-identical, the energy and virial sums agree to their rounding."""
    s = CASES["nacl_13824"]()
    runs = []
    for env, apw in (("256", "16"), ("1024", "0"), ("256", "0")):
        monkeypatch.setenv("GB_PAIR_NT", env)
        monkeypatch.setenv("GB_PAIR_APW", apw)
        gpu_lib.init(s, precision=precision)
        gpu_lib.relocate()
        gpu_lib.link_cell_pairs(want_list=False)
        e, st = gpu_lib.two_body_forces()
        runs.append((e, st, gpu_lib.download(), gpu_lib.pair_counts()))
    monkeypatch.delenv("GB_PAIR_NT", raising=False)
    monkeypatch.delenv("GB_PAIR_APW", raising=False)
    ea, sa, a, ca = runs[0]
    tol = 1e-12 if precision == 0 else 1e-10
    for eb, sb, b, cb in runs[1:]:
        assert ca[5] == 1 and cb[5] == 1  # the sorted-position kernels ran
        for k in ("fx", "fy", "fz"):
            assert np.array_equal(a[k], b[k]), k
        for k in ea:
            assert abs(eb[k] - ea[k]) <= tol * max(abs(ea[k]), 1.0), k
        assert np.abs(sb - sa).max() <= tol * np.abs(sa).max()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_deferred_step_scalars_match_per_step_readback(gpu_lib, monkeypatch, precision):
    """The NVE loop that reads each step's energy, virial and stress sums after its last
    step gives the same per-step scalars and the same trajectory as the loop that reads
    them at every step."""
    s = systems.nacl_melt(16)
    out = []
    for env in ("0", "1"):
        monkeypatch.setenv("GB_MD_DEFER", env)
        gpu_lib.init(s, precision=precision)
        gpu_lib.start()
        st = gpu_lib.md_vv(30)
        out.append((st, gpu_lib.download()))
    monkeypatch.delenv("GB_MD_DEFER", raising=False)
    (sa, a), (sb, b) = out
    assert any(x.list_rebuilt for x in sa)
    assert [x.list_rebuilt for x in sa] == [x.list_rebuilt for x in sb]
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    for x, y in zip(sa, sb):
        for f in ("engcpe_rc", "vircpe_rc", "engcpe_rl", "vircpe_rl", "engvdw", "virvdw", "engke"):
            assert getattr(x, f) == getattr(y, f), f
        assert list(x.stress) == list(y.stress) and list(x.strkin) == list(y.strkin)


@pytest.mark.parametrize("precision,overlap", [(0, "1"), (1, "1"), (2, "1"), (0, "0")],
                         ids=["fp64", "mixed", "fp64_native", "fp64_one_stream"])
def test_graph_steps_match_launched_steps(gpu_lib, monkeypatch, precision, overlap):
    """The NVE loop's steps replayed as CUDA graphs (stage 1 with the list check; a step
    without rebuild, captured again after each rebuild) run the same kernels as the loop
    that launches them one by one: the same trajectory and step scalars bit for bit, and
    the same kernel count; with SPME on the side stream (forked and joined inside the
    graph) or on one stream.  The all-native-FP64 form sums its pair forces with FP64
    atomics, whose order varies from run to run with or without graphs: it is compared
    at the MD-trajectory bar (1e-9) instead."""
    s = systems.nacl_melt(16)
    out = []
    monkeypatch.setenv("GB_OVERLAP", overlap)
    for env in ("0", "1"):
        monkeypatch.setenv("GB_GRAPHS", env)
        gpu_lib.init(s, precision=precision)
        gpu_lib.start()
        l0 = gpu_lib.lib.gb_kernel_launches()
        st = gpu_lib.md_vv(40)
        out.append((st, gpu_lib.download(), gpu_lib.lib.gb_kernel_launches() - l0))
    monkeypatch.delenv("GB_GRAPHS", raising=False)
    monkeypatch.delenv("GB_OVERLAP", raising=False)
    (sa, a, na), (sb, b, nb) = out
    assert sum(x.list_rebuilt for x in sa) >= 2
    assert [x.list_rebuilt for x in sa] == [x.list_rebuilt for x in sb]
    exact = precision != 2
    for k in a:
        if exact:
            assert np.array_equal(a[k], b[k]), k
        else:
            assert np.abs(a[k] - b[k]).max() <= 1e-9 * np.abs(b[k]).max(), k
    for x, y in zip(sa, sb):
        for f in ("engcpe_rc", "vircpe_rc", "engcpe_rl", "vircpe_rl", "engvdw", "virvdw", "engke"):
            if exact:
                assert getattr(x, f) == getattr(y, f), f
            else:
                assert getattr(x, f) == pytest.approx(getattr(y, f), rel=1e-9), f
        if exact:
            assert list(x.stress) == list(y.stress) and list(x.strkin) == list(y.strkin)
    assert na == nb


@pytest.mark.parametrize("name", ["nacl_4096", "water_5184"])
def test_fp32_tile_spread_matches_fixed_point_spread(gpu_lib, oracle_lib, monkeypatch, name):
    """FP32 grids (mixed form) spread by the atomic-free tile kernel, each brick's atoms in
    atom-index order, against the fixed-point atomic spread (GB_SPREAD_FIX=1): both within
    the mixed form's bound of the FP64 oracle, within FP32 rounding of each other, and the
    tile spread gives the same bits on a second call."""
    s = CASES[name]()
    oracle_lib.init(s)
    oracle_lib.relocate()
    er, _, _ = oracle_lib.ewald_spme_forces()
    b = oracle_lib.download()
    runs = {}
    for mode, env in (("fix", "1"), ("tile", "0")):
        monkeypatch.setenv("GB_SPREAD_FIX", env)
        gpu_lib.init(s, precision=1)
        gpu_lib.relocate()
        runs[mode] = [(gpu_lib.ewald_spme_forces(), gpu_lib.download()) for _ in range(2)]
    monkeypatch.delenv("GB_SPREAD_FIX", raising=False)
    for mode, r in runs.items():
        (ed, _, _), a = r[0]
        assert force_rms_rel(a, b) <= 1e-5, mode
        assert ed == pytest.approx(er, rel=1e-6), mode
    (t0, a0), (t1, a1) = runs["tile"]
    assert t0[0] == t1[0]
    for k in ("fx", "fy", "fz"):
        assert np.array_equal(a0[k], a1[k]), k
    assert force_rms_rel(runs["fix"][0][1], a0) <= 2e-6


def _pinned_rows(n, rows):
    """`rows` float64 arrays of n values, views into one pinned host allocation."""
    torch = pytest.importorskip("torch")
    block = torch.zeros((rows, n), dtype=torch.float64).pin_memory().numpy()
    return [block[k] for k in range(rows)], block


def test_state_transfer_mapped_and_copy_paths(gpu_lib, monkeypatch):
    """gb_upload_state / gb_download_state with pinned caller buffers (one transfer kernel
    each way, reading and writing the mapped host memory) against the cudaMemcpyAsync path
    (GB_MAPPED_COPY=0) and against pageable buffers: the same bits after 5 MD steps, and a
    non-finite position rejected on both paths."""
    s = systems.nacl_melt(16)
    n = s.natms
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("GB_MAPPED_COPY", mode)
        gpu_lib.init(s)
        src, _ = _pinned_rows(n, 6)
        for k, v in zip(("x", "y", "z", "vx", "vy", "vz"), src):
            v[:] = getattr(s, k)
        gpu_lib.upload(*src)
        gpu_lib.start()
        gpu_lib.md_vv(5)
        rows, _ = _pinned_rows(n, 9)
        pinned = gpu_lib.download(out=dict(zip(gpu_lib.STATE_KEYS, rows)))
        pageable = gpu_lib.download()
        for k in gpu_lib.STATE_KEYS:
            assert np.array_equal(pinned[k], pageable[k]), (mode, k)
        out[mode] = {k: v.copy() for k, v in pinned.items()}
        bad, _ = _pinned_rows(n, 3)
        for k, v in zip(("x", "y", "z"), bad):
            v[:] = getattr(s, k)
        bad[2][n - 1] = np.inf
        with pytest.raises(Exception) as e:
            gpu_lib.upload(*bad)
        assert getattr(e.value, "code", None) == -5, mode
    monkeypatch.delenv("GB_MAPPED_COPY", raising=False)
    for k in gpu_lib.STATE_KEYS:
        assert np.array_equal(out["1"][k], out["0"][k]), k


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name", ["nacl_4096", "water_5184"])
def test_spme_side_stream_matches_one_stream(gpu_lib, monkeypatch, name, precision):
    """SPME on the second stream while the pair kernel runs (the default) against both on
    one stream (GB_OVERLAP=0): the same bits for forces, energies, virials and stress, at
    the start-up force call and over 10 MD steps (per-step read-back and deferred)."""
    s = CASES[name]()
    out = {}
    for mode in ("0", "1"):
        monkeypatch.setenv("GB_OVERLAP", mode)
        gpu_lib.init(s, precision=precision)
        e, st = gpu_lib.start()
        f0 = gpu_lib.download()
        steps = gpu_lib.md_vv(10)
        out[mode] = (e, st, f0, steps, gpu_lib.download())
    monkeypatch.delenv("GB_OVERLAP", raising=False)
    a, b = out["0"], out["1"]
    assert a[0] == b[0]
    assert np.array_equal(a[1], b[1])
    for k in gpu_lib.STATE_KEYS:
        assert np.array_equal(a[2][k], b[2][k]), k
        assert np.array_equal(a[4][k], b[4][k]), k
    for x, y in zip(a[3], b[3]):
        for f in ("engcpe_rc", "vircpe_rc", "engcpe_rl", "vircpe_rl", "engcpe_ex", "vircpe_ex", "engvdw", "virvdw",
                  "engke"):
            assert getattr(x, f) == getattr(y, f), f
        assert list(x.stress) == list(y.stress)
