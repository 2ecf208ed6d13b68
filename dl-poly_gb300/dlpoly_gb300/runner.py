"""Standalone NVE run from DL_POLY input files, on the GPU path.

    python -m dlpoly_gb300.runner emit <workload> <dir> [--steps N] [--stats N]
    python -m dlpoly_gb300.runner run <dir> [--steps N]

'emit' writes a seeded synthetic workload as CONFIG, FIELD, CONTROL (new-style keys)
and the raw arrays (arrays.npz).  'run' reads CONTROL, FIELD, CONFIG and the optional
GBCONTROL (gb_precision, gb_mts_k, gb_mts_tol, gb_mts_train, gb_device), runs
time_run steps through the C-ABI (gb_init, gb_relocate, gb_list_build, gb_forces,
gb_md_run) and writes what the reference's NVE run writes for this path:

  STATIS  one record every stats_frequency steps, step 0 included (statistics.F90:933)
  REVCON  levcfg 2 every data_dump_frequency steps and at the end (configuration.F90:2446)
  REVIVE  accumulators at the same points (system.F90:1831, unformatted branch)

'ensemble nve' or 'ensemble nvt' with ensemble_method berendsen, hoover or
langevin selects the VV stages (gb_set_ensemble).  'restart noscale' keeps the
CONFIG velocities, 'scale' rescales them to the temperature key, 'continue' keeps
them and reads REVIVE (statistics and the thermostat's chi_t and cint).  'clean' draws new
Maxwell-Boltzmann velocities from a fixed seed (the reference's random stream is
not reproduced) and is refused for systems with constraints.

Mean-square displacements (the per-type amsd columns of STATIS) come from positions
read back at each STATIS record: displacements are unwrapped by the minimum image of
the motion between records, and the value is held between records.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time as _time

import numpy as np

from . import dlpoly_io as io
from . import systems
from .systems import BOLTZ

WORKLOADS = {
    "nacl_4096": (lambda: systems.nacl_melt(16), 1500.0),
    "nacl_175616": (lambda: systems.nacl_melt(56, kmax=160), 1500.0),
    "nacl_262144": (lambda: systems.nacl_melt(64), 1500.0),
    "water_1536": (lambda: systems.spce_water(8), 300.0),
    "water_98304": (lambda: systems.spce_water(32), 300.0),
    "eam_6912": (lambda: systems.eam_alloy(12), 600.0),
    "eam_256000": (lambda: systems.eam_alloy(40), 600.0),
}


def emit(workload: str, directory: str, steps: int = 100, stats_every: int = 10, gb: dict | None = None):
    make, temp = WORKLOADS[workload]
    s = make()
    return io.emit_inputs(s, directory, steps, temp, stats_every, gb)


def _kinetic(s, vel):
    m = s.weight[:, None] * (s.lfrzn == 0)[:, None]
    engke = 0.5 * float(np.sum(m * vel * vel))
    strkin = np.einsum("na,nb->ab", m * vel, vel).reshape(-1)          # kinstress, kinetics.F90:218
    return engke, strkin


def _set_velocities(s, ctl, degfre):
    restart = ctl.get("restart", "clean")
    temp = float(ctl.get("temperature", 0.0))
    vel = np.stack([s.vx, s.vy, s.vz], 1)
    if restart == "clean":
        if s.ntcons:
            raise NotImplementedError("restart clean draws velocities: not done for constrained systems; "
                                      "write velocities into CONFIG and use 'restart noscale' or 'scale'")
        rng = np.random.Generator(np.random.PCG64(20240601))
        vel = rng.standard_normal((s.natms, 3)) * np.sqrt(BOLTZ * max(temp, 0.0) / s.weight)[:, None]
        vel[s.lfrzn != 0] = 0.0
        mass = s.weight * (s.lfrzn == 0)
        vel -= (mass[:, None] * vel).sum(0) / max(mass.sum(), 1e-300)
    if restart in ("clean", "scale") and temp > 0.0:
        engke, _ = _kinetic(s, vel)
        target = 0.5 * degfre * BOLTZ * temp
        if engke > 0.0:
            vel *= math.sqrt(target / engke)
    s.vx, s.vy, s.vz = (np.ascontiguousarray(vel[:, k]) for k in range(3))


def _min_image(d, cell):
    c = np.asarray(cell).reshape(3, 3)
    f = d @ np.linalg.inv(c)
    f -= np.round(f)
    return f @ c


def run(directory: str, steps: int | None = None, lib=None, quiet: bool = False) -> dict:
    """Run the inputs in `directory`; returns a summary dict (also printed as JSON)."""
    j = lambda name: os.path.join(directory, name)
    ctl = io.read_control(j("CONTROL"))
    gb = io.read_control(j("GBCONTROL"), io.GB_KEYS) if os.path.exists(j("GBCONTROL")) else {}
    fld = io.read_field(j(ctl.get("io_file_field", "FIELD")))
    cfg = io.read_config(j(ctl.get("io_file_config", "CONFIG")))
    s = io.system_from_files(cfg, fld, ctl, tabeam=j("TABEAM") if fld.metal else None)
    nrun = int(ctl.get("time_run", 0)) if steps is None else int(steps)
    st_every = int(ctl.get("stats_frequency", 0))
    dump_every = int(ctl.get("data_dump_frequency", 1000))
    stats = io.Statistics(s, units=fld.units, stack_size=int(ctl.get("stack_size", 0)))
    _set_velocities(s, ctl, stats.degfre)
    nstep0, time0 = 0, 0.0
    restart = ctl.get("restart", "clean")
    revive = j(ctl.get("io_file_revive", "REVIVE"))
    if restart == "continue" and os.path.exists(revive):
        info = stats.read_revive(revive)
        nstep0, time0 = info["nstep"], info["time"]
    elif restart == "continue":
        nstep0, time0 = cfg.step, cfg.time

    if lib is None:
        from . import load
        lib = load()
    precision = {"fp64": 0, "mixed": 1}[gb.get("gb_precision", "fp64")]
    lib.init(s, precision=precision, device=int(gb.get("gb_device", 0)))
    ens = io.ensemble_from_control(ctl)
    if ens["kind"] != "nve":
        lib.set_ensemble(ens["kind"], ens["temp"], ens["tau_t"], ens["chi"], ens.get("seed"), stats.degfre)
        if restart == "continue" and os.path.exists(revive):
            lib.set_thermostat_state(info["chi_t"], info["cint"])
    lib.set_step(nstep0)
    if int(gb.get("gb_mts_k", 1)) > 1:
        lib.mts_config(int(gb["gb_mts_k"]), float(gb.get("gb_mts_tol", 1e-4)), int(gb.get("gb_mts_train", 0)))
    e0, s0 = lib.start()
    st0 = lib.download()
    pos_prev = np.stack([st0["x"], st0["y"], st0["z"]], 1)
    disp = np.zeros_like(pos_prev)
    vel0 = np.stack([st0["vx"], st0["vy"], st0["vz"]], 1)
    engke0, strkin0 = _kinetic(s, vel0)

    statis_path = j(ctl.get("io_file_statis", "STATIS"))
    mode = "a" if (restart == "continue" and os.path.exists(statis_path)) else "w"
    fh = open(statis_path, mode)
    if mode == "w":
        fh.write(stats.header(cfg.title or s.name))

    def amsd_now(pos):
        nonlocal pos_prev, disp
        disp += _min_image(pos - pos_prev, s.cell)
        pos_prev = pos
        r2 = np.sum(disp * disp, 1) * (s.lfrzn == 0)
        return np.bincount(s.ltype - 1, weights=r2, minlength=s.ntypes)

    step0 = dict(e0, engke=engke0, vircon=0.0, stress=s0, strkin=strkin0, strcon=np.zeros(9))
    if s.eam:
        me = lib.metal_energies()
        step0.update(engmet=me["engmet"] + me["engden"], virmet=me["virmet"] + me["virden"])
    if restart != "continue":                 # a continued run already recorded its first step
        stats.collect(nstep0, step0, s.cell, amsd=np.zeros(s.ntypes))
        if st_every > 0 and nstep0 % st_every == 0:
            fh.write(stats.statis_record(nstep0, time0))

    def dump(nstep, tnow, last_stats):
        d = lib.download()
        frc = np.stack([d["fx"], d["fy"], d["fz"]], 1)
        snap = io.Config(title=cfg.title or s.name, levcfg=2, imcon=cfg.imcon, cell=s.cell,
                         names=[s.type_names[t - 1] for t in s.ltype], index=np.arange(1, s.natms + 1),
                         pos=np.stack([d["x"], d["y"], d["z"]], 1),
                         vel=np.stack([d["vx"], d["vy"], d["vz"]], 1), frc=frc,
                         step=nstep, tstep=s.tstep, time=tnow)
        io.write_config(j(ctl.get("io_file_revcon", "REVCON")), snap)
        th = lib.thermostat_state()
        stats.write_revive(revive, s.rcut, s.natms, nstep, s.tstep, tnow, time0,
                           last_stats.get("strcon", np.zeros(9)), last_stats["stress"],
                           rbin=float(ctl.get("rdf_binsize", 0.05)), chi_t=th["chi_t"], cint=th["cint"])

    t_wall = _time.perf_counter()
    nstep, done = nstep0, 0
    last = step0
    amsd = np.zeros(s.ntypes)
    list_rebuilds = shake = rattle = 0
    while done < nrun:
        chunk = nrun - done
        for every in (st_every, dump_every):
            if every > 0:
                chunk = min(chunk, every - (nstep % every))
        out = lib.md_vv(chunk)
        for k, rec in enumerate(out):
            nstep += 1
            d = {f: getattr(rec, f) for f in ("engcpe_rc", "vircpe_rc", "engcpe_rl", "vircpe_rl", "engcpe_ex",
                                              "vircpe_ex", "engvdw", "virvdw", "engke", "vircon", "engmet",
                                              "virmet")}
            d["stress"] = np.array(rec.stress[:])
            d["strkin"] = np.array(rec.strkin[:])
            d["strcon"] = np.array(rec.strcon[:])
            d["consv"] = rec.consv
            list_rebuilds += rec.list_rebuilt
            shake += rec.shake_iters
            rattle += rec.rattle_iters
            recorded = st_every > 0 and nstep % st_every == 0
            if recorded and k == len(out) - 1:
                dd = lib.download()
                amsd = amsd_now(np.stack([dd["x"], dd["y"], dd["z"]], 1))
            stats.collect(nstep, d, s.cell, amsd=amsd)
            if recorded:
                fh.write(stats.statis_record(nstep, time0 + (nstep - nstep0) * s.tstep))
            last = d
        done += len(out)
        if dump_every > 0 and nstep % dump_every == 0 and done < nrun:
            dump(nstep, time0 + (nstep - nstep0) * s.tstep, last)
    wall = _time.perf_counter() - t_wall
    fh.close()
    dump(nstep, time0 + (nstep - nstep0) * s.tstep, last)
    summary = {
        "system": s.name, "natms": s.natms, "steps": nrun, "final_step": nstep,
        "wall_s": wall, "atom_steps_per_s": s.natms * nrun / wall if wall > 0 else None,
        "precision": gb.get("gb_precision", "fp64"),
        "engtot": float(stats.stpval[1]), "temperature": float(stats.stpval[2]),
        "list_rebuilds": list_rebuilds, "shake_iters": shake, "rattle_iters": rattle,
    }
    if not quiet:
        print(json.dumps(summary))
    return summary


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m dlpoly_gb300.runner")
    sub = ap.add_subparsers(dest="cmd", required=True)
    e = sub.add_parser("emit", help="write a synthetic workload as DL_POLY inputs")
    e.add_argument("workload", choices=sorted(WORKLOADS))
    e.add_argument("directory")
    e.add_argument("--steps", type=int, default=100)
    e.add_argument("--stats", type=int, default=10)
    e.add_argument("--precision", choices=["fp64", "mixed"], default=None)
    e.add_argument("--mts-k", type=int, default=None)
    r = sub.add_parser("run", help="run CONTROL/FIELD/CONFIG in a directory")
    r.add_argument("directory")
    r.add_argument("--steps", type=int, default=None)
    a = ap.parse_args(argv)
    if a.cmd == "emit":
        gb = {}
        if a.precision:
            gb["gb_precision"] = a.precision
        if a.mts_k:
            gb["gb_precision"] = "mixed"
            gb["gb_mts_k"] = a.mts_k
        emit(a.workload, a.directory, a.steps, a.stats, gb or None)
    else:
        run(a.directory, a.steps)


if __name__ == "__main__":
    sys.exit(main())
