#!/usr/bin/env python
"""Benchmark of the GB300 DL_POLY per-timestep force and update path.

Metric: atom-steps/s (and ns/day at dt = 2 fs) of the NVE velocity-Verlet MD
step: VV stage 1, conditional Verlet-list rebuild (link cells + halo images),
SPME reciprocal forces (order-8 B-splines, 3-D FFT + influence function),
real-space vdW + erfc-Coulomb pair forces, VV stage 2.

Default workload (one GPU): the 262,144-ion NaCl-like melt (64^3 rock-salt
sites, 180.48 A box, SPME grid 192^3, order 8, rc 12 A, skin 1 A), seeded
synthetic start at 1500 K.  The headline `value` is the plain FP64 form; the
line's "forms" object holds every form of the same workload measured the same
way: "mixed" (FP32 arithmetic, 2^40 fixed-point forces) with its RMS and max
force error against FP64 at the same positions, and "mts_k4" / "mts_k8" (the
learned multiple-time-step form on the mixed path, network trained online for
--mts-train steps before timing, fallback bound 1e-4) with the errors its
checks measured.  The working set (Verlet list ~0.8 GB, grids ~0.5 GB)
exceeds the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb|reference]
                    [--form fp64|mixed|mts_k4|mts_k8] [--no-compare]

N > 1 (torchrun, one rank per GPU) runs N independent replicas: the path does
not shard (one GPU per DL_POLY rank); value = total atom-steps / max rank time.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "dl-poly_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

from dlpoly_gb300 import systems  # noqa: E402

DT_PS = 0.002
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")


def workload(name):
    if name == "nacl_262144":
        return systems.nacl_melt(64), "NaCl melt 262,144 ions, box 180.48 A, SPME 192^3 p=8, rc 12 A, skin 1 A"
    if name == "nacl_175616":  # profiling size: working set above the L2, a few GB on the device
        return (systems.nacl_melt(56, kmax=160),
                "NaCl melt 175,616 ions, box 157.92 A, SPME 160^3 p=8, rc 12 A, skin 1 A")
    if name == "nacl_4096":
        return systems.nacl_melt(16), "NaCl melt 4,096 ions, box 45.12 A, SPME 48^3 p=8, rc 12 A, skin 1 A"
    if name == "water_98304":
        return (systems.spce_water(32),
                "SPC/E-style water 32,768 molecules (98,304 atoms), box 99.3 A, SPME 100^3 p=8, rc 10 A, SHAKE/RATTLE")
    if name == "eam_256000":
        return (systems.eam_alloy(40),
                "fcc Cu-Ni alloy 256,000 atoms, box 142.6 A, tabulated Sutton-Chen EAM (5,000-point tables), "
                "rc 7 A, skin 0.5 A, no electrostatics")
    if name == "eam_6912":
        return systems.eam_alloy(12), "fcc Cu-Ni alloy 6,912 atoms, tabulated Sutton-Chen EAM, rc 7 A"
    raise SystemExit(f"unknown workload {name}")


# ------------------------------------------------------------------ dist
class Dist:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ------------------------------------------------------------ clock samples
class Clocks:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for k, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(k)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------- roofline
def kernel_work(name, s, cnt, form):
    """Algorithmic (flops, bytes) of one launch of a kernel (fixed counting convention)."""
    N = s.natms
    K = s.kmax
    K3 = K[0] * K[1] * K[2]
    p = s.nsplines
    esz = 8 if form.startswith("fp64") else 4
    P_list, P_rc = cnt
    if name == "pair_forces":
        return 10.0 * P_list + 55.0 * P_rc, N * (24 + 8 + 4 + 24) + 4.0 * P_list
    if name == "fft_x_fwd" or name == "fft_x_inv":
        return 5.0 * K3 * math.log2(K[0]), K3 * (esz + 2 * esz)
    if name == "fft_y":
        return 5.0 * K3 * math.log2(K[1]), K3 * 2 * (2 * esz)
    if name == "fft_z_conv":
        return 10.0 * K3 * math.log2(K[2]) + 6.0 * K3, K3 * (2 * 2 * 2 * esz + 2 * esz)
    if name == "spme_spread":
        return 2.0 * p ** 3 * N, N * (16 + 3 * p * esz) + K3 * esz
    if name == "spme_gather":
        return 8.0 * p ** 3 * N, K3 * esz + N * (32 + 24)
    if name == "spme_prep":
        return 3.0 * N * (p * p + 3 * p), N * (32 + 3 * p * esz + 16)
    if name == "list_pairs":
        return 10.0 * P_list, 4.0 * P_list + N * 48
    if name == "metal_density":   # distance + up to two density interpolations per entry; rho atomics
        return 10.0 * P_list + 24.0 * P_rc, N * (24 + 4 + 8 + 8) + 4.0 * P_list
    if name == "metal_forces":    # distance + three table interpolations + force, virial, stress
        return 10.0 * P_list + 60.0 * P_rc, N * (24 + 4 + 8 + 24) + 4.0 * P_list + 8.0 * P_rc
    return None


# DRAM bytes (read + write) per half-list entry of the pair kernels, from one
# ncu capture each on the 175,616-ion melt (the 262,144-ion launch is too large
# for a full-section capture); traffic grows with the list, so the bench scales
# it by this launch's list entries.
MEASURED_TRAFFIC = {
    ("pair_forces", "fp64"): ((223.553536e6 + 4.797952e6) / 40368337,
                              "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_pair_sorted<0, 4, 1024> on nacl_175616 "
                              "(profiles/pair_sorted_df64_nacl175616.md), scaled by half-list entries"),
    ("pair_forces", "fp64_native"): ((200.795648e6 + 3.779072e6) / 40368337,
                                     "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_pair_fp64 on nacl_175616 "
                                     "(profiles/pair_fp64_nacl175616.md), scaled by half-list entries"),
    ("pair_forces", "mixed"): ((219.659264e6 + 6.057216e6) / 40368337,
                               "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_pair_sorted<1, 4, 256> on nacl_175616 "
                               "(profiles/pair_sorted_mixed_nacl175616.md), scaled by half-list entries"),
    ("metal_forces", "fp64"): ((131.494144e6 + 4.494848e6) / 19246179,
                               "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_metal_forces on eam_256000 "
                               "(profiles/metal_kernels_eam256000.md), scaled by half-list entries"),
}


# Warp instructions executed per half-list entry by the double-float pair kernel (ncu
# smsp__inst_executed.sum of one launch on the 175,616-ion melt over its list
# entries).  That kernel runs on the FP32/ALU pipes and is bound by instruction
# issue, so its roofline is issue slots: 4 warp instructions per clock per SM.
MEASURED_INST = {
    ("pair_forces", "fp64"): (601732163 / 40368337,
                              "ncu smsp__inst_executed.sum of k_pair_sorted<0, 4, 1024> on nacl_175616 "
                              "(profiles/pair_sorted_df64_nacl175616.md), scaled by half-list entries"),
}


def read_peaks():
    try:
        return json.load(open(PEAKS_FILE))
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------ CPU baseline
def cpu_sample(s, steps_max, budget_s):
    """Time the FP64 oracle (OpenMP, all host cores) on the same workload."""
    import oracle

    o = oracle.load(openmp=True)
    cores = os.cpu_count() or 1
    o.lib.orc_set_threads(cores)
    o.init(s)
    o.start()
    t0 = time.perf_counter()
    o.md_vv(1)
    t1 = time.perf_counter()
    per = t1 - t0
    n = max(1, min(steps_max, int(budget_s / max(per, 1e-6))))
    t0 = time.perf_counter()
    o.md_vv(n)
    dt = time.perf_counter() - t0
    o.finalize()
    return s.natms * n / dt, cores, n, dt


def run_reference(args, dist):
    s, desc = workload(args.workload)
    if dist.rank != 0:
        return
    steps_cap = max(1, args.steps)
    budget = float(os.environ.get("GB_REF_BUDGET_S", "240"))
    val, cores, n, dt = cpu_sample(s, steps_cap, budget_s=budget)
    line = {
        "impl": "reference",
        "metric": "atom-steps/s",
        "value": val,
        "unit": "atom-steps/s",
        "n_gpus": args.gpus,
        "steps": n,
        "steps_requested": args.steps,
        "steps_match": n == args.steps,
        "time_budget_s": budget,
        "warmup": 1,
        "warmup_note": "one untimed MD step (the CPU path has no compilation or cache state beyond it); "
                       "the timed steps are --steps unless they would exceed time_budget_s",
        "ms_per_step": 1e3 * dt / n,
        "ns_per_day": (n / dt) * DT_PS * 86400 / 1000,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": desc, "form": "fp64", "natms": s.natms},
        "cpu_baseline": {"value": val, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{n} full MD steps of the same workload after one untimed step "
                                   "(C++ FP64 restatement with OpenMP; the Fortran reference has no compiler here)"},
        "e2e": {"value": val, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU arm
# form: (precision, MTS k).  fp64 evaluates the pair loop and SPME in double-float (FP64
# accuracy on the FP32 pipes); fp64_native runs the same path in FP64 instructions.
FORMS = {"fp64": (0, 1), "fp64_native": (2, 1), "mixed": (1, 1), "mts_k4": (1, 4), "mts_k8": (1, 8)}
MTS_TOL = 1e-4


def force_error(lib, L):
    """RMS and max |F_mixed - F_fp64| / RMS|F_fp64| at the current positions."""
    L.gb_set_precision.argtypes = [ctypes.c_int]
    lib.two_body_forces()
    a = lib.download()
    L.gb_set_precision(0)
    lib.two_body_forces()
    b = lib.download()
    L.gb_set_precision(1)
    Fa = np.stack([a["fx"], a["fy"], a["fz"]], 1)
    Fb = np.stack([b["fx"], b["fy"], b["fz"]], 1)
    rms = np.sqrt((Fb ** 2).sum(1).mean())
    return float(np.sqrt(((Fa - Fb) ** 2).sum(1).mean()) / rms), float(np.abs(Fa - Fb).max() / rms)


def measure(lib, L, s, form, args, dist, device, steps, detail):
    """Initialise, warm up (and train the MTS network), then time `steps` MD steps."""
    precision, k = FORMS[form]
    lib.init(s, precision=precision, device=device)
    lib.start()
    train = 0
    t_train = 0.0
    if k > 1:
        train = args.mts_train
        lib.mts_config(k, MTS_TOL, train)
        steps = k * max(1, -(-steps // k))  # whole MTS cycles
        t0 = time.perf_counter()
        lib.md_vv(train)
        t_train = time.perf_counter() - t0
    lib.md_vv(max(3, args.warmup))
    # ---- timed region: `runs` times K resident MD steps; the line reports the median run.
    # SPME runs on the library's second stream while the pair kernel runs, so per-kernel
    # times are taken afterwards in a one-stream pass of K more steps (gb_set_overlap(0)),
    # where every kernel has the whole GPU: the kernel table and the roofline use that pass.
    clocks = Clocks(device) if detail else None
    spans, walls, stats_all, launches = [], [], [], 0
    for _ in range(max(1, args.runs)):
        dist.barrier()
        l0 = L.gb_kernel_launches()
        w0 = time.perf_counter()
        stats = lib.md_vv(steps)
        w1 = time.perf_counter()
        l1 = L.gb_kernel_launches()
        tm = (ctypes.c_double * 8)()
        L.gb_last_timings(tm, 8)
        dist.barrier()
        spans.append(dist.max(tm[5] * 1e-3))
        walls.append(w1 - w0)
        stats_all += stats
        launches += l1 - l0
    clk = clocks.stop() if clocks else None
    order = sorted(range(len(spans)), key=lambda r: spans[r])
    med = order[len(order) // 2]
    tmax = spans[med]
    L.gb_set_overlap(0)
    L.gb_profile(1)
    lib.md_vv(steps)
    tm = (ctypes.c_double * 8)()
    L.gb_last_timings(tm, 8)
    one_stream_ms = tm[5] / steps
    names = ctypes.create_string_buffer(32 * 32)
    ms = (ctypes.c_double * 32)()
    nl = (ctypes.c_int64 * 32)()
    nk = L.gb_profile_read(names, ms, nl, 32)
    L.gb_profile(0)
    L.gb_set_overlap(1)
    prof = {}
    for j in range(nk):
        nm = names.raw[32 * j:32 * (j + 1)].split(b"\0")[0].decode()
        if nl[j]:
            prof[nm] = (ms[j], int(nl[j]))
    cnt = (ctypes.c_int64 * 3)()
    L.gb_pair_counts(cnt, 3)
    P_list, P_rc = int(cnt[0]), int(cnt[1])  # both forms walk the half list
    stats = stats_all
    out = {"value": dist.world * s.natms * steps / tmax, "ms_per_step": tmax * 1e3 / steps,
           "ns_per_day": (steps / tmax) * DT_PS * 86400 / 1000, "steps": steps,
           "runs": len(spans), "ms_per_step_runs": [t * 1e3 / steps for t in spans],
           "spread_rel": (max(spans) - min(spans)) / tmax,
           "one_stream_ms_per_step": one_stream_ms,
           "list_rebuilds": sum(x.list_rebuilt for x in stats) / len(spans)}
    if precision == 1 and k == 1:
        out["force_err_rms"], out["force_err_max"] = force_error(lib, L)
    if k > 1:
        m = lib.mts_stats()
        out["mts"] = {"k": k, "tol": MTS_TOL, "train_steps": train, "train_wall_s": t_train,
                      "full_spme_steps_timed": sum(x.mts_full for x in stats), "coarse_grid": int(m["coarse_k"]),
                      "checked_err_last": m["last_err"], "checked_err_max": m["err_max"],
                      "err_without_network": m["err_no_network"], "err_stale_force": m["err_stale"],
                      "fallback_entries": int(m["n_fallback"]), "in_fallback": bool(m["in_fallback"])}
    if prof:
        out["kernels_ms_per_step"] = {nm: v[0] / steps for nm, v in prof.items()}
    return out, dict(stats=stats, prof=prof, P=(P_list, P_rc), launches=launches, clk=clk, wall=sum(walls),
                     tmax=tmax, runs=len(spans))


KB_INTERNAL = 0.831446261815324  # Boltzmann constant in DL_POLY internal energy units (10 J/mol) per K


def run_drift(args):
    """NVE energy drift per form: slope of a linear fit to the total energy (after the first
    tenth of the run, and after MTS training; MTS forms use the full-SPME steps, whose energies
    are exact), in kT per ns per atom.  --drift-dt, --drift-skin and --drift-seeds repeat the
    measurement over time steps, Verlet skins and seeds of the synthetic start."""
    import dlpoly_gb300 as gb

    _, desc = workload(args.drift_workload)
    temp = 1500.0 if args.drift_workload.startswith("nacl") else 300.0
    lib = gb.load()
    out = {"mode": "nve_drift", "workload": desc, "steps": args.drift_steps, "temperature_K": temp, "runs": []}
    for dt_fs in [float(v) for v in args.drift_dt.split(",")]:
        for skin in [float(v) for v in args.drift_skin.split(",")]:
            for seed in [int(v) for v in args.drift_seeds.split(",")]:
                s = drift_system(args.drift_workload, seed)
                s.tstep = dt_fs * 1e-3
                s.rpad = skin
                nsteps = int(round(args.drift_steps * 2.0 / dt_fs))  # the same simulated time
                for form in args.drift_forms.split(","):
                    rec = drift_one(lib, s, form, nsteps, temp, args)
                    rec.update({"form": form, "dt_fs": dt_fs, "skin_A": skin, "seed": seed, "steps": nsteps})
                    out["runs"].append(rec)
    lib.finalize()
    print(json.dumps(out), flush=True)


def drift_system(name, seed):
    if name == "nacl_4096":
        return systems.nacl_melt(16, seed=seed)
    if name == "nacl_262144":
        return systems.nacl_melt(64, seed=seed)
    if name == "water_98304":
        return systems.spce_water(32, seed=seed)
    raise SystemExit(f"no drift system {name}")


def drift_one(lib, s, form, nsteps, temp, args):
    precision, k = FORMS[form]
    lib.init(s, precision=precision)
    lib.start()
    train = 0
    if k > 1:
        train = min(args.drift_train, nsteps // 2)
        lib.mts_config(k, MTS_TOL, train)
    E, full = [], []
    t0 = time.perf_counter()
    done = 0
    rebuilds = 0
    while done < nsteps:
        st = lib.md_vv(min(1000, nsteps - done))
        done += len(st)
        for x in st:
            E.append(x.engcpe_rc + x.engcpe_rl + x.engcpe_ex + x.engvdw + x.engke)
            full.append(x.mts_full)
            rebuilds += x.list_rebuilt
    wall = time.perf_counter() - t0
    E = np.array(E)
    tps = s.tstep
    idx = np.arange(len(E))
    sel = idx >= max(train + 10, len(E) // 10)
    if k > 1:
        sel &= np.array(full, bool)
    slope = np.polyfit(idx[sel] * tps, E[sel], 1)[0]  # energy units per ps
    rec = {"drift_kT_per_ns_per_atom": float(slope * 1000.0 / (KB_INTERNAL * temp * s.natms)),
           "energy_rel_std": float(np.std(E[sel]) / abs(np.mean(E[sel]))), "wall_s": wall,
           "list_rebuilds": int(rebuilds)}
    if k > 1:
        m = lib.mts_stats()
        rec["mts"] = {"k": k, "train_steps": train, "checked_err_last": m["last_err"],
                      "checked_err_max": m["err_max"], "err_without_network": m["err_no_network"],
                      "inner_steps": int(m["n_inner"]), "fallback_entries": int(m["n_fallback"])}
    return rec


def run_gb(args, dist):
    import dlpoly_gb300 as gb

    s, desc = workload(args.workload)
    precision = FORMS[args.form][0]
    lib = gb.load()
    L = lib.lib
    L.gb_profile.argtypes = [ctypes.c_int]
    L.gb_set_overlap.argtypes = [ctypes.c_int]
    L.gb_profile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64),
                                  ctypes.c_int]
    L.gb_pair_counts.argtypes = [ctypes.POINTER(ctypes.c_int64), ctypes.c_int]
    L.gb_fp64_peak_tflops.restype = ctypes.c_double
    device = dist.local
    # the other forms of the same workload, each measured the same way
    forms = {}
    if args.compare:
        for f in FORMS:
            if s.eam and f != "fp64":
                continue  # metals run in the FP64 form only
            if f != args.form:
                forms[f], _ = measure(lib, L, s, f, args, dist, device, args.steps, detail=False)
    head, det = measure(lib, L, s, args.form, args, dist, device, args.steps, detail=True)
    forms[args.form] = head
    stats, prof, (P_list, P_rc), clk, tmax = det["stats"], det["prof"], det["P"], det["clk"], det["tmax"]
    l0, l1, w0, w1 = 0, det["launches"] // det["runs"], 0.0, det["wall"] / det["runs"]
    steps = head["steps"]
    value = head["value"]
    rebuilds = head["list_rebuilds"]
    # ---- end to end through the C-ABI with host buffers (H2D state, D2H state + forces)
    ke = max(1, min(args.steps, 10))
    try:
        import torch

        def pinned(a):
            t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
            return t.numpy()
    except Exception:  # noqa: BLE001
        def pinned(a):
            return np.ascontiguousarray(a)
    d = lib.download()
    host = {k: pinned(v) for k, v in d.items()}
    dist.barrier()
    e0 = time.perf_counter()
    for _ in range(ke):
        lib.upload(host["x"], host["y"], host["z"], host["vx"], host["vy"], host["vz"])
        lib.md_vv(1)
        lib.download(out=host)
    e1 = time.perf_counter()
    emax = dist.max(e1 - e0)
    e2e = {"value": dist.world * s.natms * ke / emax, "unit": "atom-steps/s",
           "h2d_bytes_per_step": 6 * 8 * s.natms, "d2h_bytes_per_step": 9 * 8 * s.natms,
           "steps": ke, "path": "gb_upload_state + gb_md_run(1) + gb_download_state per step"}
    # ---- roofline of the dominant kernel
    peaks = read_peaks()
    hbm = peaks.get("hbm_gbs")
    fp64_peak = L.gb_fp64_peak_tflops()
    dom = max(prof.items(), key=lambda kv: kv[1][0])[0] if prof else None
    roof = None
    kernels = {}
    for nm, (t_ms, n_l) in prof.items():
        w = kernel_work(nm, s, (P_list, P_rc), args.form)
        entry = {"ms_total": t_ms, "launches": n_l, "ms_per_launch": t_ms / n_l,
                 "share": t_ms / max(1e-9, sum(v[0] for v in prof.values()))}
        if w:
            fl, by = w
            sec = t_ms / n_l * 1e-3
            entry["tflops"] = fl / sec / 1e12
            entry["gbs"] = by / sec / 1e9
        kernels[nm] = entry
    if dom and kernel_work(dom, s, (P_list, P_rc), args.form):
        fl, by = kernel_work(dom, s, (P_list, P_rc), args.form)
        sec = prof[dom][0] / prof[dom][1] * 1e-3
        inst = MEASURED_INST.get((dom, args.form)) if precision == 0 else None
        fp64_view = None
        if args.form.startswith("fp64") and fp64_peak and fp64_peak > 0:
            fp64_view = {"achieved": fl / sec / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": fl / sec / 1e12 / fp64_peak,
                         "peak_source": "FP64 DFMA loop measured in this run"}
        if inst:
            try:
                import torch
                nsm = torch.cuda.get_device_properties(device).multi_processor_count
            except Exception:  # noqa: BLE001
                nsm = 152
            mhz = (clk or {}).get("sm_mhz") or 2070.0
            peak_i = nsm * 4 * mhz * 1e6 / 1e9
            ach_i = inst[0] * P_list / sec / 1e9
            roof = {"bound": "issue", "kernel": dom, "achieved": ach_i, "peak": peak_i, "unit": "Gwarp-inst/s",
                    "frac": ach_i / peak_i, "traffic": None,
                    "peak_source": f"4 warp instructions per clock per SM x {nsm} SMs x {mhz:.0f} MHz "
                                   "(median SM clock sampled in the timed region)",
                    "inst_source": inst[1],
                    "fp64_view": fp64_view,
                    "hbm_view": {"achieved": by / sec / 1e9, "peak": hbm, "unit": "GB/s",
                                 "frac": (by / sec / 1e9) / hbm if hbm else None}}
        elif args.form.startswith("fp64") and fp64_peak and fp64_peak > 0 and fl / by > fp64_peak * 1e3 / (hbm or 6751.1):
            roof = {"bound": "fp64", "kernel": dom, "achieved": fl / sec / 1e12, "peak": fp64_peak,
                    "unit": "TFLOP/s", "frac": fl / sec / 1e12 / fp64_peak, "traffic": None,
                    "peak_source": "FP64 DFMA loop measured in this run (MEASURED_PEAKS.json has no FP64 figure)",
                    "hbm_view": {"achieved": by / sec / 1e9, "peak": hbm, "unit": "GB/s",
                                 "frac": (by / sec / 1e9) / hbm if hbm else None}}
        else:
            roof = {"bound": "hbm", "kernel": dom, "achieved": by / sec / 1e9, "peak": hbm or 6800.0, "unit": "GB/s",
                    "frac": (by / sec / 1e9) / (hbm or 6800.0), "traffic": None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs" if hbm else "fallback 6.8 TB/s"}
        roof["algorithmic"] = {"flops_per_launch": fl, "bytes_per_launch": by, "launch_ms": sec * 1e3}
        tr = MEASURED_TRAFFIC.get((dom, args.form if args.form.startswith("fp64") else "mixed"))
        if tr:
            roof["traffic"] = tr[0] * P_list
            roof["traffic_source"] = tr[1]
    # the all-FP64 form's pair kernel against the FP64 pipe (DFMA peak measured in this run)
    nat = forms.get("fp64_native")
    if nat and fp64_peak and fp64_peak > 0 and "pair_forces" in nat.get("kernels_ms_per_step", {}):
        fl, by = kernel_work("pair_forces", s, (P_list, P_rc), "fp64_native")
        t_pair = nat["kernels_ms_per_step"]["pair_forces"] * 1e-3
        nat["roofline"] = {"bound": "fp64", "kernel": "pair_forces (k_pair_fp64)",
                           "achieved": fl / t_pair / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
                           "frac": fl / t_pair / 1e12 / fp64_peak,
                           "peak_source": "FP64 DFMA loop measured in this run",
                           "flops_per_launch": fl, "launch_ms": t_pair * 1e3}
    # speed ratios between the forms of this workload (same steps, same clock record)
    ratios = {}
    for a, b in (("mixed", "fp64_native"), ("mixed", "fp64"), ("fp64", "fp64_native"), ("mts_k4", "mixed"),
                 ("mts_k8", "mixed")):
        if a in forms and b in forms:
            ratios[f"{a}_over_{b}"] = forms[a]["value"] / forms[b]["value"]
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        try:
            v, cores, n, dt = cpu_sample(s, 2, budget_s=30.0)
            cpu = {"value": v, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                   "sample": f"{n} full MD steps of the same workload, C++ FP64 oracle with OpenMP on {cores} host threads"}
        except Exception as e:  # noqa: BLE001
            cpu = {"value": None, "error": str(e)}
    lib.finalize()
    if dist.rank != 0:
        return
    line = {
        "metric": "atom-steps/s",
        "value": value,
        "unit": "atom-steps/s",
        "n_gpus": dist.world,
        "steps": steps,
        "warmup": max(3, args.warmup),
        "ms_per_step": tmax * 1e3 / steps,
        "ns_per_day": (steps / tmax) * DT_PS * 86400 / 1000,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        # fp64: pair loop and SPME in double-float (two f32 per value, FP64-level accuracy),
        # list, integration and constraints in f64; mixed: f32 arithmetic, i64 fixed-point sums
        "dtype": {0: "df64+f64", 2: "f64"}.get(precision, "f32+i64"),
        "data": "synthetic (seeded lattice + Maxwell-Boltzmann start)",
        "config": {"workload": desc, "form": args.form, "natms": s.natms, "dt_fs": 2.0,
                   "list_rebuilds_in_timed_steps": rebuilds, "parallelism": "replicas" if dist.world > 1 else "single",
                   "l2": "working set > 129 MB L2 (list ~%.0f MB), no flush" % (4.0 * P_list / 1e6)},
        "forms": forms,
        "ratios": ratios,
        "runs": det["runs"],
        "ms_per_step_runs": head["ms_per_step_runs"],
        "spread_rel": head["spread_rel"],
        "e2e": e2e,
        "gpu_launches": int(l1 - l0),
        "clocks": clk,
        "roofline": roof,
        "kernels": kernels,
        "kernels_timing": "CUDA events per phase in a one-stream pass of the same number of steps after the timed "
                          "runs (SPME and the pair kernel on one stream: gb_set_overlap(0)); the timed runs overlap "
                          "SPME on a second stream with the pair kernel",
        "one_stream_ms_per_step": head["one_stream_ms_per_step"],
        "pairs": {"list_entries": P_list, "within_rc": P_rc},
        "wall_s_timed": w1 - w0,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--runs", type=int, default=3, help="timed runs of --steps steps each; the line reports the median")
    ap.add_argument("--impl", default="gb", choices=["gb", "reference"])
    ap.add_argument("--form", default="fp64", choices=list(FORMS))
    ap.add_argument("--workload", default="nacl_262144",
                    choices=["nacl_262144", "nacl_175616", "nacl_4096", "water_98304", "eam_256000", "eam_6912"])
    ap.add_argument("--mts-train", type=int, default=2000,
                    help="MD steps of online training (SPME every step) before the learned-MTS forms are timed")
    ap.add_argument("--no-compare", dest="compare", action="store_false",
                    help="time only --form (default: every form of the workload, --form is the headline)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--drift", action="store_true", help="NVE energy drift per form instead of the throughput line")
    ap.add_argument("--drift-workload", default="nacl_4096", choices=["nacl_4096", "nacl_262144", "water_98304"])
    ap.add_argument("--drift-steps", type=int, default=10000)
    ap.add_argument("--drift-train", type=int, default=2000)
    ap.add_argument("--drift-forms", default="fp64,mixed,mts_k4,mts_k8")
    ap.add_argument("--drift-dt", default="2", help="time steps in fs (comma list); steps scale to equal time")
    ap.add_argument("--drift-skin", default="1", help="Verlet skins in Angstrom (comma list)")
    ap.add_argument("--drift-seeds", default="1234", help="seeds of the synthetic start (comma list)")
    ap.add_argument("--emit", metavar="DIR", default=None,
                    help="write the workload as DL_POLY CONFIG/FIELD/CONTROL plus raw arrays and exit")
    args = ap.parse_args()
    if args.emit:
        from dlpoly_gb300 import dlpoly_io

        s, _ = workload(args.workload)
        temp = 1500.0 if args.workload.startswith("nacl") else 300.0
        dlpoly_io.emit_inputs(s, args.emit, steps=args.steps, temperature=temp, stats_every=1)
        print(json.dumps({"emitted": args.emit, "workload": args.workload, "natms": s.natms}))
        return
    if args.drift:
        run_drift(args)
        return
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_gb(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
