"""Seeded synthetic systems in the shapes of the benchmark workloads.

No dataset is involved: the ionic melts and the water box are generated from a
seed, in DL_POLY internal units (Angstrom, ps, amu, 10 J/mol, charges in e).

Workloads
---------
nacl_melt(n_side)      rock-salt lattice of n_side^3 sites, spacing 2.82 A, +/-1 e,
                       +/-0.2 A uniform jitter, Maxwell-Boltzmann 1500 K;
                       12-6 LJ with Lorentz-Berthelot mixing; SPME rc 12 A.
                       n_side=16 -> 4,096 ions (48^3 grid); n_side=64 -> 262,144 ions (192^3).
spce_water(n_side)     rigid 3-site water on an n_side^3 cubic lattice at 1.0 g/cm^3,
                       random orientations, 300 K; O-O LJ only; SHAKE/RATTLE bonds;
                       rc 10 A.  n_side=32 -> 32,768 molecules (98,304 atoms, 100^3 grid).
eam_alloy(n_side)      random fcc Cu-Ni alloy with Sutton-Chen EAM tables (TABEAM form),
                       no charges; rc 7 A.  n_side=12 -> 6,912 atoms; n_side=40 -> 256,000.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

BOLTZ = 0.831451115  # constants.F90:104, 10 J/mol/K
KJ = 100.0           # kJ/mol in internal energy units (constants.F90:114)


class GbParams(ctypes.Structure):
    """ctypes mirror of gb_params (include/gb300_dlpoly.h)."""

    _fields_ = [
        ("cell", ctypes.c_double * 9),
        ("rcut", ctypes.c_double),
        ("rpad", ctypes.c_double),
        ("rvdw", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("epsq", ctypes.c_double),
        ("tstep", ctypes.c_double),
        ("shake_tol", ctypes.c_double),
        ("pdplnc", ctypes.c_double),
        ("kmax", ctypes.c_int32 * 3),
        ("nsplines", ctypes.c_int32),
        ("spline_pad", ctypes.c_int32),
        ("vdw_direct", ctypes.c_int32),
        ("shake_maxit", ctypes.c_int32),
        ("max_list", ctypes.c_int32),
        ("max_exclude", ctypes.c_int32),
        ("mxatms", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("ntypes", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("mxnode", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 5),
    ]


class GbStepStats(ctypes.Structure):
    """ctypes mirror of gb_step_stats."""

    _fields_ = [
        ("engcpe_rc", ctypes.c_double), ("vircpe_rc", ctypes.c_double),
        ("engcpe_rl", ctypes.c_double), ("vircpe_rl", ctypes.c_double),
        ("engcpe_ex", ctypes.c_double), ("vircpe_ex", ctypes.c_double),
        ("engvdw", ctypes.c_double), ("virvdw", ctypes.c_double),
        ("engke", ctypes.c_double), ("vircon", ctypes.c_double),
        ("stress", ctypes.c_double * 9), ("strkin", ctypes.c_double * 9),
        ("strcon", ctypes.c_double * 9),
        ("consv", ctypes.c_double),
        ("engmet", ctypes.c_double), ("virmet", ctypes.c_double),
        ("list_rebuilt", ctypes.c_int32), ("shake_iters", ctypes.c_int32),
        ("rattle_iters", ctypes.c_int32), ("mts_full", ctypes.c_int32),
    ]


def ewald_alpha(precision: float, rcut: float) -> float:
    """Ewald alpha from 'spme_precision' as control.F90:1707-1709 derives it."""
    tol = math.sqrt(abs(math.log(precision * rcut)))
    return math.sqrt(abs(math.log(precision * rcut * tol))) / rcut


@dataclass
class System:
    """Topology, parameters and initial state of one workload."""

    name: str
    cell: np.ndarray            # (9,) rows of the cell matrix
    ltype: np.ndarray           # int32 (N,), 1-based
    chge: np.ndarray            # float64 (N,)
    weight: np.ndarray          # float64 (N,)
    lfrzn: np.ndarray           # int32 (N,)
    vdw_prm: np.ndarray         # float64 (nkey*3,) (kind, eps, sigma)
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    rcut: float
    rpad: float
    alpha: float
    kmax: tuple
    ntypes: int
    nsplines: int = 8
    tstep: float = 0.002
    shake_tol: float = 1.0e-8
    listcon: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    prmcon: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    max_exclude: int = 0
    list_excl: np.ndarray | None = None
    vdw_direct: int = 0
    type_names: tuple = ()      # site name per 1-based type (FIELD 'atoms' records)
    epsq: float = 1.0           # relative dielectric constant
    shake_maxit: int = 250
    # tabulated EAM metal tables (TABEAM order): list of dicts with kind ('pair', 'dens',
    # 'embe'), types (t1, t2), start, finish and values (energies in internal units)
    eam: list | None = None
    metal_listed: np.ndarray | None = None   # per type-pair key: listed in FIELD 'metal'

    @property
    def natms(self) -> int:
        return int(self.ltype.shape[0])

    @property
    def ntcons(self) -> int:
        return int(self.listcon.shape[0] // 3)

    def volume(self) -> float:
        c = self.cell.reshape(3, 3)
        return abs(float(np.linalg.det(c)))

    def params(self, precision: int = 0, max_list: int | None = None, device: int = 0) -> GbParams:
        p = GbParams()
        p.device = device
        for k in range(9):
            p.cell[k] = float(self.cell[k])
        p.rcut = self.rcut
        p.rpad = self.rpad
        p.rvdw = self.rcut
        p.alpha = self.alpha
        p.epsq = self.epsq
        p.tstep = self.tstep
        p.shake_tol = self.shake_tol
        p.pdplnc = 50.0
        for d in range(3):
            p.kmax[d] = int(self.kmax[d])
        p.nsplines = self.nsplines
        # bounds.F90:1249: padded spline halo, ~2% over the order
        p.spline_pad = self.nsplines + int(math.ceil(0.02 * self.nsplines))
        p.vdw_direct = self.vdw_direct
        p.shake_maxit = self.shake_maxit
        dens = self.natms / self.volume()
        rcx = self.rcut + self.rpad
        # bounds.F90:907 style capacity: density * (7.5/3) * pi * rcx^3
        p.max_list = int(max_list if max_list is not None else round(dens * 2.5 * math.pi * rcx**3) + 64)
        p.max_exclude = max(self.max_exclude, 1)
        L = min(self.cell[0], self.cell[4], self.cell[8])
        w = L / max(1, int(L / (rcx + 1e-6)))
        grow = ((L + 2.0 * w) / L) ** 3
        p.mxatms = int(self.natms * grow * 1.15) + 4096
        p.precision = precision
        p.ntypes = self.ntypes
        return p

    def excl_array(self, p: GbParams) -> np.ndarray:
        ld = p.max_exclude + 1
        out = np.zeros(ld * self.natms, np.int32)
        if self.list_excl is not None:
            src = self.list_excl
            m = src.shape[1]
            full = np.zeros((self.natms, ld), np.int32)
            full[:, :m] = src
            out[:] = full.reshape(-1)
        return out


def _maxwell(rng, mass, temp):
    sig = np.sqrt(BOLTZ * temp / mass)
    v = rng.standard_normal((mass.shape[0], 3)) * sig[:, None]
    p = (v * mass[:, None]).sum(0) / mass.sum()
    return v - p[None, :]


def nacl_melt(n_side: int = 16, seed: int = 1234, spacing: float = 2.82, temp: float = 1500.0,
              rcut: float = 12.0, kmax: int | None = None, jitter: float = 0.2) -> System:
    """NaCl-like ionic melt on an n_side^3 rock-salt lattice (cubic box n_side*spacing)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = n_side * spacing
    g = np.arange(n_side)
    ix, iy, iz = np.meshgrid(g, g, g, indexing="ij")
    ix, iy, iz = ix.ravel(), iy.ravel(), iz.ravel()
    n = ix.size
    cation = ((ix + iy + iz) % 2) == 0
    pos = np.stack([ix, iy, iz], 1).astype(np.float64) * spacing + 0.5 * spacing - 0.5 * L
    pos += rng.uniform(-jitter, jitter, size=pos.shape)
    ltype = np.where(cation, 1, 2).astype(np.int32)
    chge = np.where(cation, 1.0, -1.0)
    weight = np.where(cation, 22.99, 35.45)
    v = _maxwell(rng, weight, temp)
    eps = {1: 0.40 * KJ, 2: 0.42 * KJ}
    sig = {1: 2.50, 2: 4.40}
    prm = []
    for a in (1, 2):
        for b in range(1, a + 1):
            e = math.sqrt(eps[a] * eps[b])          # Lorentz-Berthelot, ffield.F90:4125-4128
            s = 0.5 * (sig[a] + sig[b])
            prm += [1.0, e, s]
    alpha = ewald_alpha(1.0e-6, rcut)
    if kmax is None:
        kmax = {16: 48, 64: 192}.get(n_side, 2 * int(round(0.25 + L * alpha * 3.0 / math.pi)))
    cell = np.array([L, 0, 0, 0, L, 0, 0, 0, L], np.float64)
    return System(name=f"nacl_melt_{n}", cell=cell, ltype=ltype, chge=chge, weight=weight,
                  lfrzn=np.zeros(n, np.int32), vdw_prm=np.array(prm, np.float64),
                  x=pos[:, 0].copy(), y=pos[:, 1].copy(), z=pos[:, 2].copy(),
                  vx=v[:, 0].copy(), vy=v[:, 1].copy(), vz=v[:, 2].copy(),
                  rcut=rcut, rpad=1.0, alpha=alpha, kmax=(kmax, kmax, kmax), ntypes=2,
                  type_names=("Na", "Cl"))


def _random_rotations(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z); R[:, 0, 1] = 2 * (x * y - z * w); R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w); R[:, 1, 1] = 1 - 2 * (x * x + z * z); R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w); R[:, 2, 1] = 2 * (y * z + x * w); R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def spce_water(n_side: int = 32, seed: int = 4321, temp: float = 300.0, rcut: float = 10.0,
               box: float | None = None, kmax: int | None = None) -> System:
    """Rigid 3-site SPC/E-style water on an n_side^3 lattice at 1.0 g/cm^3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nmol = n_side ** 3
    mO, mH = 15.9994, 1.008
    if box is None:
        # 1.0 g/cm^3: volume per molecule = M / (N_A * rho) in A^3
        box = (nmol * (mO + 2 * mH) / 0.6022140857) ** (1.0 / 3.0)
    L = box
    a = L / n_side
    g = np.arange(n_side)
    ix, iy, iz = np.meshgrid(g, g, g, indexing="ij")
    com = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], 1) * a + 0.5 * a - 0.5 * L
    theta = math.radians(109.47)
    dOH = 1.0
    dHH = 2.0 * dOH * math.sin(0.5 * theta)
    # body frame: O at origin, H in the xz plane, then shift to the centre of mass
    h1 = np.array([dOH * math.sin(0.5 * theta), 0.0, dOH * math.cos(0.5 * theta)])
    h2 = np.array([-dOH * math.sin(0.5 * theta), 0.0, dOH * math.cos(0.5 * theta)])
    body = np.stack([np.zeros(3), h1, h2])
    cm = (mO * body[0] + mH * body[1] + mH * body[2]) / (mO + 2 * mH)
    body = body - cm
    R = _random_rotations(rng, nmol)
    sites = np.einsum("nij,sj->nsi", R, body) + com[:, None, :]
    pos = sites.reshape(-1, 3)
    n = pos.shape[0]
    ltype = np.tile(np.array([1, 2, 2], np.int32), nmol)
    chge = np.tile(np.array([-0.8476, 0.4238, 0.4238]), nmol)
    weight = np.tile(np.array([mO, mH, mH]), nmol)
    v = _maxwell(rng, weight, temp)
    # constraints: (type, gi, gj), 1-based global ids; types 1 = O-H, 2 = H-H
    base = 3 * np.arange(nmol) + 1
    listcon = np.stack([
        np.stack([np.ones(nmol), base, base + 1], 1),
        np.stack([np.ones(nmol), base, base + 2], 1),
        np.stack([2 * np.ones(nmol), base + 1, base + 2], 1),
    ], 1).reshape(-1).astype(np.int32)
    prmcon = np.array([dOH, dHH], np.float64)
    v = _rattle_project(v, pos, weight, listcon, L)
    excl = np.zeros((n, 3), np.int32)
    mol = np.arange(n) // 3
    for s in range(3):
        others = [t for t in range(3) if t != s]
        idx = np.arange(nmol) * 3 + s
        excl[idx, 0] = 2
        excl[idx, 1] = 3 * mol[idx] + others[0] + 1
        excl[idx, 2] = 3 * mol[idx] + others[1] + 1
    # vdW keys: (1,1)=O-O LJ, (2,1) none, (2,2) none
    prm = [1.0, 0.650 * KJ, 3.166, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0]
    alpha = ewald_alpha(1.0e-6, rcut)
    if kmax is None:
        kmax = {32: 100}.get(n_side, 2 * int(round(0.25 + L * alpha * 3.0 / math.pi)))
    cell = np.array([L, 0, 0, 0, L, 0, 0, 0, L], np.float64)
    return System(name=f"spce_water_{n}", cell=cell, ltype=ltype, chge=chge, weight=weight,
                  lfrzn=np.zeros(n, np.int32), vdw_prm=np.array(prm, np.float64),
                  x=pos[:, 0].copy(), y=pos[:, 1].copy(), z=pos[:, 2].copy(),
                  vx=v[:, 0].copy(), vy=v[:, 1].copy(), vz=v[:, 2].copy(),
                  rcut=rcut, rpad=1.0, alpha=alpha, kmax=(kmax, kmax, kmax), ntypes=2,
                  listcon=listcon, prmcon=prmcon, max_exclude=2, list_excl=excl,
                  type_names=("OW", "HW"))


def _rattle_project(v, pos, mass, listcon, L):
    """Remove bond-stretching velocity components so the start obeys the constraints.

    The three constraints of each molecule (consecutive in listcon) are solved
    exactly: v' = v - M^-1 G^T lam with (G M^-1 G^T) lam = G v, G the bond
    gradients d_k . (v_i - v_j)."""
    lc = listcon.reshape(-1, 3)
    nmol = lc.shape[0] // 3
    i = (lc[:, 1] - 1).reshape(nmol, 3)
    j = (lc[:, 2] - 1).reshape(nmol, 3)
    d = pos[i] - pos[j]
    d -= L * np.round(d / L)
    atoms = 3 * np.arange(nmol)[:, None] + np.arange(3)[None, :]  # molecule-local atoms
    li = i - atoms[:, :1]
    lj = j - atoms[:, :1]
    G = np.zeros((nmol, 3, 3, 3))  # constraint k, atom a, component
    for kk in range(3):
        G[np.arange(nmol), kk, li[:, kk], :] += d[:, kk, :]
        G[np.arange(nmol), kk, lj[:, kk], :] -= d[:, kk, :]
    minv = 1.0 / mass[atoms]  # (nmol, 3)
    Gf = G.reshape(nmol, 3, 9)
    Minv = np.repeat(minv, 3, axis=1)  # (nmol, 9)
    A = np.einsum("nkc,nc,nlc->nkl", Gf, Minv, Gf)
    vm = v[atoms].reshape(nmol, 9)
    rhs = np.einsum("nkc,nc->nk", Gf, vm)
    lam = np.linalg.solve(A, rhs[..., None])[..., 0]
    vm = vm - Minv * np.einsum("nkc,nk->nc", Gf, lam)
    out = v.copy()
    out[atoms.reshape(-1)] = vm.reshape(nmol * 3, 3)
    return out


def lj_pair(eps: float = 1.0, sigma: float = 2.0, r: float = 1.0, box: float = 40.0) -> System:
    """Two neutral atoms at distance r (the vdW known-answer fixture)."""
    cell = np.array([box, 0, 0, 0, box, 0, 0, 0, box], np.float64)
    return System(name="lj_pair", cell=cell, ltype=np.array([1, 1], np.int32),
                  chge=np.zeros(2), weight=np.ones(2), lfrzn=np.zeros(2, np.int32),
                  vdw_prm=np.array([1.0, eps, sigma]), x=np.array([0.0, r]), y=np.zeros(2),
                  z=np.zeros(2), vx=np.zeros(2), vy=np.zeros(2), vz=np.zeros(2), rcut=10.0,
                  rpad=0.5, alpha=0.3, kmax=(16, 16, 16), ntypes=1, vdw_direct=1,
                  type_names=("Ar",))


# Sutton-Chen parameters (Sutton and Chen, Phil. Mag. Lett. 61 (1990) 139): epsilon [eV],
# a [A], n, m, c for the two species of the synthetic alloy
SUTTON_CHEN = {"Cu": (1.2382e-2, 3.61, 9, 6, 39.432), "Ni": (1.5707e-2, 3.52, 9, 6, 39.432)}
EV = 9648.530821   # eV in internal energy units (constants.F90:112)


def _taper(r, r_on, rc):
    """1 below r_on, (1 - x^2)^2 with x = (r - r_on)/(rc - r_on) up to rc, 0 beyond:
    value and slope continuous at both ends."""
    x = np.clip((r - r_on) / (rc - r_on), 0.0, 1.0)
    return (1.0 - x * x) ** 2


def eam_tables(species=("Cu", "Ni"), rc: float = 7.0, r_on: float = 6.0, r_min: float = 1.5,
               ngrid: int = 5000, rho_max: float = 400.0):
    """Sutton-Chen EAM sampled as TABEAM tables: pair V_ab = eps_ab (a_ab/r)^n, density
    rho_b(r) = (a_b/r)^m (contributed by a neighbour of species b), embedding
    F_a(rho) = -c_a eps_a sqrt(rho); eps_ab = sqrt(eps_a eps_b), a_ab = (a_a + a_b)/2.
    Pair and density taper smoothly to zero between r_on and rc."""
    r = np.linspace(r_min, rc, ngrid)
    rho = np.linspace(0.0, rho_max, ngrid)
    tabs = []
    nt = len(species)
    for ia in range(nt):
        for ib in range(ia + 1):
            ea, aa, n, m, _ = SUTTON_CHEN[species[ia]]
            eb, ab, _, _, _ = SUTTON_CHEN[species[ib]]
            e, a = math.sqrt(ea * eb), 0.5 * (aa + ab)
            v = e * (a / r) ** n * _taper(r, r_on, rc) * EV
            tabs.append({"kind": "pair", "types": (ia + 1, ib + 1), "start": r_min, "finish": rc, "values": v})
    for ia in range(nt):
        _, a, _, m, _ = SUTTON_CHEN[species[ia]]
        tabs.append({"kind": "dens", "types": (ia + 1, ia + 1), "start": r_min, "finish": rc,
                     "values": (a / r) ** m * _taper(r, r_on, rc)})
    for ia in range(nt):
        e, _, _, _, c = SUTTON_CHEN[species[ia]]
        tabs.append({"kind": "embe", "types": (ia + 1, ia + 1), "start": 0.0, "finish": rho_max,
                     "values": -c * e * np.sqrt(rho) * EV})
    return tabs


def eam_alloy(n_side: int = 12, seed: int = 2468, lattice: float = 3.565, frac_ni: float = 0.5,
              temp: float = 600.0, jitter: float = 0.05, rc: float = 7.0) -> System:
    """Random fcc Cu-Ni alloy on n_side^3 cubic cells (4 sites each) with Sutton-Chen
    EAM tables; no charges and no vdW.  n_side = 12 -> 6,912 atoms; 40 -> 256,000."""
    rng = np.random.Generator(np.random.PCG64(seed))
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.arange(n_side)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    pos = ((cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) + 0.25) * lattice
    L = n_side * lattice
    pos = pos - 0.5 * L + rng.uniform(-jitter, jitter, pos.shape)
    n = pos.shape[0]
    ltype = np.where(rng.random(n) < frac_ni, 2, 1).astype(np.int32)
    weight = np.where(ltype == 1, 63.546, 58.6934)
    v = _maxwell(rng, weight, temp)
    cell = np.array([L, 0, 0, 0, L, 0, 0, 0, L], np.float64)
    return System(name=f"eam_cuni_{n}", cell=cell, ltype=ltype, chge=np.zeros(n), weight=weight,
                  lfrzn=np.zeros(n, np.int32), vdw_prm=np.zeros(9), x=pos[:, 0].copy(),
                  y=pos[:, 1].copy(), z=pos[:, 2].copy(), vx=v[:, 0].copy(), vy=v[:, 1].copy(),
                  vz=v[:, 2].copy(), rcut=rc, rpad=0.5, alpha=0.3, kmax=(16, 16, 16), ntypes=2,
                  type_names=("Cu", "Ni"), eam=eam_tables(("Cu", "Ni"), rc=rc, r_on=rc - 1.0),
                  metal_listed=np.ones(3, np.int32))
