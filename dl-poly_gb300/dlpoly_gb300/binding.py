"""ctypes binding of the path's C-ABI (include/gb300_dlpoly.h).

`PathLib` wraps one shared library whose exports follow the gb_* signatures
under a name prefix.  The GB300 library exports them as gb_*; the method names
mirror the reference's Fortran routines that each export replaces, so a test
reads like the reference's own call sequence:

    relocate()            relocate_particles + set_halo_particles (halo.F90:153)
    link_cell_pairs()     neighbours.F90:356
    two_body_forces()     drivers.F90:655-786 (SPME + pair loop)
    ewald_spme_forces()   ewald_spole.F90:244
    nve_0_vv(stage)       nve.F90:38 (with apply_shake / apply_rattle)
    md_vv(nsteps)         drivers.F90:2059 resident loop

Every non-zero status raises `PathError` carrying the DL_POLY error code.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int, c_int32, c_int64, c_void_p

import numpy as np

from .systems import GbParams, GbStepStats, System

_d = POINTER(c_double)
_i = POINTER(c_int32)


class PathError(RuntimeError):
    def __init__(self, code: int, where: str, text: str = ""):
        super().__init__(f"{where}: status {code} {text}".strip())
        self.code = code


def _ptr(a, t):
    if a is None:
        return None
    return a.ctypes.data_as(t)


SIGNATURES = {
    "init": (c_int, [POINTER(GbParams), c_int, _i, _d, _d, _i, _d, c_int, _i, _d, _i]),
    "upload_state": (c_int, [_d, _d, _d, _d, _d, _d]),
    "download_state": (c_int, [_d, _d, _d, _d, _d, _d, _d, _d, _d]),
    "relocate": (c_int, []),
    "list_build": (c_int, [_i, c_int, _i]),
    "vnl_check": (c_int, [_i]),
    "refresh": (c_int, [_i]),
    "forces": (c_int, [_d, _d]),
    "spme": (c_int, [_d, _d, _d]),
    "real": (c_int, [_d, _d]),
    "vv": (c_int, [c_int, _d, _d, _i, _d, _d]),
    "md_run": (c_int, [c_int, POINTER(GbStepStats)]),
    "finalize": (None, []),
}


class PathLib:
    """One loaded implementation of the path (library + symbol prefix)."""

    def __init__(self, lib: ctypes.CDLL, prefix: str):
        self.lib = lib
        self.prefix = prefix
        self.fn = {}
        for name, (res, args) in SIGNATURES.items():
            f = getattr(lib, prefix + name)
            f.restype = res
            f.argtypes = args
            self.fn[name] = f
        self.sys: System | None = None
        self.params: GbParams | None = None

    def _call(self, name, *args):
        st = self.fn[name](*args)
        if st != 0:
            raise PathError(st, self.prefix + name, self.strerror(st))
        return st

    def strerror(self, st):
        f = getattr(self.lib, self.prefix + "strerror", None)
        if f is None:
            return ""
        f.restype = ctypes.c_char_p
        f.argtypes = [c_int]
        return (f(st) or b"").decode()

    # ---------------------------------------------------------------- set-up
    def init(self, s: System, precision: int = 0, max_list: int | None = None, device: int = 0, **overrides):
        """gb_init for system s; keyword overrides set gb_params fields (e.g. mxatms, shake_maxit)."""
        p = s.params(precision, max_list, device)
        for k, v in overrides.items():
            setattr(p, k, v)
        self.params = p
        self.sys = s
        excl = s.excl_array(p)
        lc = s.listcon.astype(np.int32) if s.ntcons else np.zeros(3, np.int32)
        pc = s.prmcon.astype(np.float64) if s.ntcons else np.zeros(1)
        self._keep = [s.ltype, s.chge, s.weight, s.lfrzn, s.vdw_prm, lc, pc, excl]
        self._call("init", ctypes.byref(p), s.natms, _ptr(s.ltype, _i), _ptr(s.chge, _d),
                   _ptr(s.weight, _d), _ptr(s.lfrzn, _i), _ptr(s.vdw_prm, _d), s.ntcons,
                   _ptr(lc, _i), _ptr(pc, _d), _ptr(excl, _i))
        self.upload(s.x, s.y, s.z, s.vx, s.vy, s.vz)
        if getattr(s, "eam", None):
            self.set_metal_eam(s.eam, s.metal_listed)

    # ------------------------------------------------ metals (tabulated EAM)
    _EAM_KIND = {"pair": 1, "dens": 2, "embe": 3}

    def set_metal_eam(self, tables, listed=None):
        """tables: dicts with kind ('pair', 'dens', 'embe'), types (t1, t2), start, finish,
        values (internal energy units), in TABEAM order."""
        k = np.array([self._EAM_KIND[t["kind"]] for t in tables], np.int32)
        t1 = np.array([t["types"][0] for t in tables], np.int32)
        t2 = np.array([t["types"][1] for t in tables], np.int32)
        ng = np.array([len(t["values"]) for t in tables], np.int32)
        st = np.array([t["start"] for t in tables], np.float64)
        fi = np.array([t["finish"] for t in tables], np.float64)
        vals = np.ascontiguousarray(np.concatenate([np.asarray(t["values"], np.float64) for t in tables]))
        lst = None if listed is None else np.ascontiguousarray(listed, np.int32)
        self._keep_eam = [k, t1, t2, ng, st, fi, vals, lst]
        code = self._opt("set_metal_eam", c_int, [c_int, _i, _i, _i, _i, _d, _d, _d, _i])(
            len(tables), _ptr(k, _i), _ptr(t1, _i), _ptr(t2, _i), _ptr(ng, _i), _ptr(st, _d), _ptr(fi, _d),
            _ptr(vals, _d), _ptr(lst, _i))
        if code != 0:
            raise PathError(code, self.prefix + "set_metal_eam", self.strerror(code))

    def metal_energies(self) -> dict:
        out = np.zeros(4)
        code = self._opt("metal_energies", c_int, [_d])(_ptr(out, _d))
        if code != 0:
            raise PathError(code, self.prefix + "metal_energies", self.strerror(code))
        return dict(zip(("engmet", "virmet", "engden", "virden"), out.tolist()))

    def metal_rho(self):
        out = np.zeros(self.sys.natms)
        code = self._opt("metal_rho", c_int, [_d])(_ptr(out, _d))
        if code != 0:
            raise PathError(code, self.prefix + "metal_rho", self.strerror(code))
        return out

    def upload(self, x, y, z, vx=None, vy=None, vz=None):
        a = [np.ascontiguousarray(v, np.float64) if v is not None else None for v in (x, y, z, vx, vy, vz)]
        self._call("upload_state", *[_ptr(v, _d) for v in a])

    STATE_KEYS = ("x", "y", "z", "vx", "vy", "vz", "fx", "fy", "fz")

    def download(self, out: dict | None = None):
        """Positions, velocities and forces; into the caller's arrays when `out` holds
        them (contiguous float64, e.g. pinned host buffers), else into new arrays."""
        n = self.sys.natms
        if out is None:
            out = {k: np.empty(n) for k in self.STATE_KEYS}
        arrs = [out[k] for k in self.STATE_KEYS]
        for a in arrs:
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != n:
                raise ValueError("download buffers must be contiguous float64 arrays of natms values")
        self._call("download_state", *[_ptr(v, _d) for v in arrs])
        return out

    # ----------------------------------------------------------- path calls
    def relocate(self):
        self._call("relocate")

    def link_cell_pairs(self, want_list: bool = True):
        p = self.params
        ld = p.max_list + 4
        out = np.zeros(ld * self.sys.natms, np.int32) if want_list else None
        need = np.zeros(1, np.int32)
        self._call("list_build", _ptr(out, _i), ld, _ptr(need, _i))
        return None if out is None else out.reshape(self.sys.natms, ld)

    def list_build_status(self):
        """Build and return (status, needed max_list) without raising."""
        p = self.params
        need = np.zeros(1, np.int32)
        st = self.fn["list_build"](None, p.max_list + 4, _ptr(need, _i))
        return st, int(need[0])

    def vnl_check(self) -> bool:
        u = np.zeros(1, np.int32)
        self._call("vnl_check", _ptr(u, _i))
        return bool(u[0])

    def refresh(self) -> bool:
        u = np.zeros(1, np.int32)
        self._call("refresh", _ptr(u, _i))
        return bool(u[0])

    def two_body_forces(self):
        e = np.zeros(8)
        s = np.zeros(9)
        self._call("forces", _ptr(e, _d), _ptr(s, _d))
        keys = ("engcpe_rc", "vircpe_rc", "engcpe_rl", "vircpe_rl", "engcpe_ex", "vircpe_ex", "engvdw", "virvdw")
        return dict(zip(keys, e)), s

    def ewald_spme_forces(self):
        e = np.zeros(1)
        v = np.zeros(1)
        s = np.zeros(9)
        self._call("spme", _ptr(e, _d), _ptr(v, _d), _ptr(s, _d))
        return float(e[0]), float(v[0]), s

    def real_space_forces(self):
        e = np.zeros(6)
        s = np.zeros(9)
        self._call("real", _ptr(e, _d), _ptr(s, _d))
        keys = ("engcpe_rl", "vircpe_rl", "engcpe_ex", "vircpe_ex", "engvdw", "virvdw")
        return dict(zip(keys, e)), s

    def nve_0_vv(self, stage: int):
        sk = np.zeros(9)
        ek = np.zeros(1)
        it = np.zeros(1, np.int32)
        vc = np.zeros(1)
        sc = np.zeros(9)
        self._call("vv", stage, _ptr(sk, _d), _ptr(ek, _d), _ptr(it, _i), _ptr(vc, _d), _ptr(sc, _d))
        return dict(strkin=sk, engke=float(ek[0]), iters=int(it[0]), vircon=float(vc[0]), strcon=sc)

    def constraints_tags(self):
        """constraints_tags (constraints.F90:438): bond vectors of the current positions."""
        st = self._opt("constraints_tags", c_int, [])()
        if st != 0:
            raise PathError(st, self.prefix + "constraints_tags", self.strerror(st))

    def apply_shake(self):
        """apply_shake (constraints.F90:1071) on the resident (unconstrained) positions."""
        it = np.zeros(1, np.int32)
        vc = np.zeros(1)
        sc = np.zeros(9)
        st = self._opt("shake", c_int, [_i, _d, _d])(_ptr(it, _i), _ptr(vc, _d), _ptr(sc, _d))
        if st != 0:
            raise PathError(st, self.prefix + "shake", self.strerror(st))
        return dict(iters=int(it[0]), vircon=float(vc[0]), strcon=sc)

    def apply_rattle(self):
        """apply_rattle with kit = 1 (constraints.F90:1032) on the resident velocities."""
        it = np.zeros(1, np.int32)
        st = self._opt("rattle", c_int, [_i])(_ptr(it, _i))
        if st != 0:
            raise PathError(st, self.prefix + "rattle", self.strerror(st))
        return int(it[0])

    def md_vv(self, nsteps: int):
        arr = (GbStepStats * max(1, nsteps))()
        self._call("md_run", nsteps, arr)
        return [arr[k] for k in range(nsteps)]

    def start(self):
        """Start-up as the reference does before md_vv: wrap, halo, list, forces."""
        self.relocate()
        self.link_cell_pairs(want_list=False)
        return self.two_body_forces()

    def finalize(self):
        self.fn["finalize"]()

    # ------------------------------------------------ learned-MTS form (CUDA only)
    def _opt(self, name, res, args):
        f = getattr(self.lib, self.prefix + name)
        f.restype = res
        f.argtypes = args
        return f

    # ------------------------------------------------ ensembles of the VV stages
    ENSEMBLES = {"nve": 0, "berendsen": 1, "nose-hoover": 2, "langevin": 3}

    def set_ensemble(self, kind, temp: float = 0.0, tau_t: float = 0.0, chi: float = 0.0, seed=None,
                     degfre: float = 0.0):
        k = self.ENSEMBLES[kind] if isinstance(kind, str) else int(kind)
        sd = None if seed is None else np.ascontiguousarray(seed, np.int32)
        st = self._opt("set_ensemble", c_int, [c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, _i,
                                               ctypes.c_double])(k, temp, tau_t, chi, _ptr(sd, _i), degfre)
        if st != 0:
            raise PathError(st, self.prefix + "set_ensemble", self.strerror(st))

    def set_step(self, nstep: int):
        self._opt("set_step", c_int, [ctypes.c_int32])(int(nstep))

    def thermostat_state(self) -> dict:
        v = np.zeros(3)
        st = self._opt("thermostat_state", c_int, [_d, _d, _d])(_ptr(v[0:1], _d), _ptr(v[1:2], _d),
                                                                _ptr(v[2:3], _d))
        if st != 0:
            raise PathError(st, self.prefix + "thermostat_state", self.strerror(st))
        return {"chi_t": float(v[0]), "cint": float(v[1]), "consv": float(v[2])}

    def set_thermostat_state(self, chi_t: float, cint: float):
        st = self._opt("set_thermostat_state", c_int, [ctypes.c_double, ctypes.c_double])(chi_t, cint)
        if st != 0:
            raise PathError(st, self.prefix + "set_thermostat_state", self.strerror(st))

    def rng_eval(self, mode: int, a, b, c):
        _l = POINTER(ctypes.c_int64)
        a, b, c = (np.ascontiguousarray(v, np.int64) for v in (a, b, c))
        out = np.zeros(a.size * (1 if mode == 0 else 3))
        st = self._opt("rng_eval", c_int, [c_int, c_int, _l, _l, _l, _d])(mode, a.size, _ptr(a, _l), _ptr(b, _l),
                                                                       _ptr(c, _l), _ptr(out, _d))
        if st != 0:
            raise PathError(st, self.prefix + "rng_eval", self.strerror(st))
        return out if mode == 0 else out.reshape(-1, 3)

    def pair_counts(self) -> list:
        """[half-list entries, pairs inside rc, list candidates decided in exact FP64,
        forward halo entries, backward halo entries, cell tiles used, second-launch tiles,
        cells per tile] of the last force evaluation and list build (GPU library only)."""
        out = np.zeros(8, np.int64)
        st = self._opt("pair_counts", c_int, [POINTER(c_int64), c_int])(_ptr(out, POINTER(c_int64)), 8)
        if st != 0:
            raise PathError(st, self.prefix + "pair_counts", self.strerror(st))
        return [int(v) for v in out]

    def mts_config(self, k: int, tol: float = 1e-4, train_steps: int = 0):
        st = self._opt("mts_config", c_int, [c_int, ctypes.c_double, c_int])(k, tol, train_steps)
        if st != 0:
            raise PathError(st, self.prefix + "mts_config", self.strerror(st))

    def mts_ablation(self, no_network: bool):
        """1: the inner steps use the coarse-grid force alone (no network)."""
        st = self._opt("mts_ablation", c_int, [c_int])(1 if no_network else 0)
        if st != 0:
            raise PathError(st, self.prefix + "mts_ablation", self.strerror(st))

    MTS_KEYS = ("last_err", "n_full", "n_inner", "n_fallback", "last_loss", "opt_steps", "err_max",
                "in_fallback", "n_checked", "md_steps", "err_no_network", "err_stale", "coarse_k")

    def mts_stats(self) -> dict:
        out = np.zeros(len(self.MTS_KEYS))
        self._opt("mts_stats", c_int, [_d, c_int])(_ptr(out, _d), len(out))
        return dict(zip(self.MTS_KEYS, out.tolist()))

    def mts_features(self, n: int):
        x = np.zeros((n, 51), np.float32)
        sc = np.zeros(52, np.float32)
        _f = POINTER(ctypes.c_float)
        st = self._opt("mts_features", c_int, [_f, c_int, _f])(_ptr(x, _f), n, _ptr(sc, _f))
        if st != 0:
            raise PathError(st, self.prefix + "mts_features", self.strerror(st))
        return x, sc

    def mlp_param_count(self) -> int:
        return int(self._opt("mlp_param_count", c_int, [])())

    def mlp_train_eval(self, x, target, params):
        _f = POINTER(ctypes.c_float)
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(target, np.float32)
        p = np.ascontiguousarray(params, np.float32)
        nb = x.shape[0]
        loss = np.zeros(1, np.float32)
        grad = np.zeros(p.size, np.float32)
        y = np.zeros((nb, 3), np.float32)
        st = self._opt("mlp_train_eval", c_int, [c_int, _f, _f, _f, _f, _f, _f])(
            nb, _ptr(x, _f), _ptr(t, _f), _ptr(p, _f), _ptr(loss, _f), _ptr(grad, _f), _ptr(y, _f))
        if st != 0:
            raise PathError(st, self.prefix + "mlp_train_eval", self.strerror(st))
        return float(loss[0]), grad, y

    def mlp_infer_eval(self, x, params):
        _f = POINTER(ctypes.c_float)
        x = np.ascontiguousarray(x, np.float32)
        p = np.ascontiguousarray(params, np.float32)
        y = np.zeros((x.shape[0], 3), np.float32)
        st = self._opt("mlp_infer_eval", c_int, [c_int, _f, _f, _f])(x.shape[0], _ptr(x, _f), _ptr(p, _f),
                                                                      _ptr(y, _f))
        if st != 0:
            raise PathError(st, self.prefix + "mlp_infer_eval", self.strerror(st))
        return y


def stats_to_dict(s: GbStepStats) -> dict:
    d = {k: getattr(s, k) for k, _ in GbStepStats._fields_ if k not in ("stress", "strkin", "strcon")}
    d["stress"] = np.array(s.stress[:])
    d["strkin"] = np.array(s.strkin[:])
    d["strcon"] = np.array(s.strcon[:])
    return d
