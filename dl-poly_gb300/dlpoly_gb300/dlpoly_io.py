"""DL_POLY input and output files: CONFIG/REVCON, FIELD, CONTROL, STATIS, REVIVE.

Each writer produces the records of the reference routine it names; each reader
accepts the free format that the reference reads (blank-separated words, '#'
comments, Fortran 'D' exponents).

  CONFIG, REVCON  write_config   configuration.F90:2446-2560 (write_config, serial branch)
                  read_config    configuration.F90:846 (read_config), :2051 (scan_config)
  FIELD           write_field / read_field   ffield.F90:390-420 (units), :455 (molecules),
                  :528 (nummols), :534 (atoms), :760 (constraints), :2347 (finish),
                  :3616 (vdw), :5295 (close)
  CONTROL         write_control / read_control   new-style 'key value [unit]' lines,
                  control.F90:4501-4600 (parse_control_file, read_control_param)
  STATIS          Statistics.collect / statis_record   statistics.F90:933-1400
  REVIVE          Statistics.write_revive / read_revive   system.F90:1831 (system_revive),
                  unformatted branch

Only what the force/update path runs is accepted.  FIELD directives for bonds,
angles, dihedrals, shells, rigid bodies, tethers, PMFs, metals and many-body
terms, and vdW forms other than 'lj', raise NotImplementedError; CONTROL keys
outside the registered set raise ValueError, as the reference stops with
'Unrecognised key'.
"""
from __future__ import annotations

import math
import re
import struct
from dataclasses import dataclass, field as dc_field

import numpy as np

from .systems import BOLTZ, System, ewald_alpha

# energy units of FIELD files, in internal units (10 J/mol): constants.F90:104,112-114
ENGUNIT = {"ev": 9648.530821, "kcal": 418.4, "kj": 100.0, "internal": 1.0, "k": BOLTZ}
STATIS_UNITS = {"ev": "electron Volts", "kcal": "kcal/mol", "kj": "kjoule/mol",
                "internal": "DL_POLY Internal UNITS (10 J/mol)", "k": "Kelvin/Boltzmann"}
PRSUNT = 1.63882576e-1     # internal pressure -> katm (constants.F90:123)


# --------------------------------------------------------------------------------------
# Fortran edit descriptors (Fw.d, Ew.d with and without 1P, Gw.d, Iw)
# --------------------------------------------------------------------------------------
def _stars(w: int) -> str:
    return "*" * w


def fmt_f(v: float, w: int, d: int) -> str:
    s = f"{v:{w}.{d}f}"
    return s if len(s) <= w else _stars(w)


def fmt_e(v: float, w: int, d: int, scale: int = 0) -> str:
    """Ew.d; scale=1 is the '1p' form (one digit before the point, d after)."""
    if not math.isfinite(v):
        return ("NaN" if v != v else ("Infinity" if v > 0 else "-Infinity")).rjust(w)
    a = abs(v)
    if scale == 1:
        mant, ex = f"{a:.{d}E}".split("E")
        ex = int(ex)
    else:
        mant, ex = f"{a:.{d - 1}E}".split("E")
        ex = int(ex) + 1 if a != 0.0 else 0
        mant = "0." + mant.replace(".", "")
    exs = f"E{ex:+03d}" if abs(ex) <= 99 else f"{ex:+04d}"
    s = ("-" if math.copysign(1.0, v) < 0 else "") + mant + exs
    return s.rjust(w) if len(s) <= w else _stars(w)


def fmt_g(v: float, w: int, d: int) -> str:
    """Gw.d: F editing with four trailing blanks where the magnitude allows, else Ew.d."""
    if not math.isfinite(v):
        return fmt_e(v, w, d)
    if v == 0.0:
        return fmt_f(v, w - 4, d - 1) + "    "
    ex = int(f"{abs(v):.{d - 1}E}".split("E")[1])   # decimal exponent after rounding to d digits
    k = ex + 1
    if 0 <= k <= d:
        return fmt_f(v, w - 4, d - k) + "    "
    return fmt_e(v, w, d)


def fmt_i(v: int, w: int) -> str:
    s = f"{int(v):{w}d}"
    return s if len(s) <= w else _stars(w)


_NOE = re.compile(r"^([+-]?(?:\d+\.?\d*|\.\d+))([+-]\d+)$")


def to_real(word: str) -> float:
    """A real in any Fortran form: 1.5, 1.5d0, 1.5E+02, 1.5+100 (3-digit exponent)."""
    w = word.strip().replace("D", "E").replace("d", "E")
    m = _NOE.match(w)
    if m:
        w = m.group(1) + "E" + m.group(2)
    return float(w)


def _records(path):
    with open(path) as fh:
        return fh.read().splitlines()


# --------------------------------------------------------------------------------------
# CONFIG / REVCON
# --------------------------------------------------------------------------------------
@dataclass
class Config:
    """One CONFIG (or REVCON) file: atom records in file order."""

    title: str
    levcfg: int
    imcon: int
    cell: np.ndarray                  # (9,) rows a, b, c
    names: list
    index: np.ndarray                 # int64 (N,), 1-based global ids
    pos: np.ndarray                   # (N, 3)
    vel: np.ndarray | None = None     # levcfg >= 1
    frc: np.ndarray | None = None     # levcfg >= 2
    step: int = 0
    tstep: float = 0.0
    time: float = 0.0

    @property
    def natms(self) -> int:
        return int(self.pos.shape[0])


def write_config(path, cfg: Config) -> None:
    """Records as write_config (configuration.F90:2446) writes them: every record is
    72 characters and a line feed; title (a72); levcfg, imcon, megatm, step (4i10) and
    tstep, time (1p,2e16.7); cell rows (3f20.10); per atom the name and index
    (a8,i10), positions, then velocities (levcfg >= 1) and forces (levcfg >= 2),
    each (3g20.10)."""
    if cfg.levcfg >= 1 and cfg.vel is None:
        raise ValueError("levcfg >= 1 needs velocities")
    if cfg.levcfg >= 2 and cfg.frc is None:
        raise ValueError("levcfg 2 needs forces")
    pad12 = " " * 12
    out = [cfg.title[:72].ljust(72),
           fmt_i(cfg.levcfg, 10) + fmt_i(cfg.imcon, 10) + fmt_i(cfg.natms, 10) + fmt_i(cfg.step, 10)
           + fmt_e(cfg.tstep, 16, 7, 1) + fmt_e(cfg.time, 16, 7, 1)]
    if cfg.imcon > 0:
        c = np.asarray(cfg.cell, np.float64)
        for r in range(3):
            out.append("".join(fmt_f(float(c[3 * r + k]), 20, 10) for k in range(3)) + pad12)
    blocks = [cfg.pos]
    if cfg.levcfg >= 1:
        blocks.append(cfg.vel)
    if cfg.levcfg >= 2:
        blocks.append(cfg.frc)
    blocks = [np.asarray(b, np.float64).tolist() for b in blocks]
    pad54 = " " * 54
    for i in range(cfg.natms):
        out.append(str(cfg.names[i])[:8].ljust(8) + fmt_i(int(cfg.index[i]), 10) + pad54)
        for b in blocks:
            r = b[i]
            out.append(fmt_g(r[0], 20, 10) + fmt_g(r[1], 20, 10) + fmt_g(r[2], 20, 10) + pad12)
    with open(path, "w") as fh:
        fh.write("\n".join(out))
        fh.write("\n")


def read_config(path) -> Config:
    """Free-format reader (read_config, configuration.F90:846): title, then
    'levcfg imcon [megatm step tstep time]', three cell rows when imcon /= 0, then per
    atom a name record 'name [index]' and levcfg+1 records of three reals.  Atoms
    are returned in index order when the indices are a permutation of 1..N."""
    rec = _records(path)
    if len(rec) < 2:
        raise ValueError(f"{path}: CONFIG needs a title and a levcfg/imcon record")
    title = rec[0][:72].rstrip()
    w = rec[1].split()
    levcfg, imcon = int(to_real(w[0])), int(to_real(w[1]))
    if levcfg not in (0, 1, 2):
        raise ValueError(f"{path}: levcfg {levcfg} not in 0..2")
    step = int(to_real(w[3])) if len(w) > 3 else 0
    tstep = to_real(w[4]) if len(w) > 4 else 0.0
    time = to_real(w[5]) if len(w) > 5 else 0.0
    k = 2
    cell = np.zeros(9)
    if imcon != 0:
        for r in range(3):
            cell[3 * r:3 * r + 3] = [to_real(x) for x in rec[k].split()[:3]]
            k += 1
    names, index, rows = [], [], [[] for _ in range(levcfg + 1)]
    while k < len(rec):
        w = rec[k].split()
        if not w:
            k += 1
            continue
        names.append(w[0][:8])
        index.append(int(to_real(w[1])) if len(w) > 1 else len(names))
        for b in range(levcfg + 1):
            vals = rec[k + 1 + b].split()
            rows[b].append([to_real(vals[0]), to_real(vals[1]), to_real(vals[2])])
        k += levcfg + 2
    index = np.asarray(index, np.int64)
    arrs = [np.asarray(r, np.float64).reshape(-1, 3) for r in rows]
    n = len(names)
    if n and np.array_equal(np.sort(index), np.arange(1, n + 1)):
        order = np.argsort(index, kind="stable")
        names = [names[i] for i in order]
        index = index[order]
        arrs = [a[order] for a in arrs]
    return Config(title=title, levcfg=levcfg, imcon=imcon, cell=cell, names=names, index=index,
                  pos=arrs[0], vel=arrs[1] if levcfg >= 1 else None,
                  frc=arrs[2] if levcfg >= 2 else None, step=step, tstep=tstep, time=time)


# --------------------------------------------------------------------------------------
# FIELD
# --------------------------------------------------------------------------------------
@dataclass
class Site:
    name: str
    mass: float
    charge: float
    freeze: int = 0


@dataclass
class MoleculeType:
    name: str
    nummols: int
    sites: list                                              # Site per atom of one molecule
    constraints: list = dc_field(default_factory=list)       # (i, j, length), 1-based local


@dataclass
class Field:
    title: str
    units: str                    # key of ENGUNIT
    molecules: list
    vdw: list                     # (name1, name2, 'lj', (epsilon [file units], sigma [A]))
    metal: list = dc_field(default_factory=list)   # (name1, name2, 'eam'): tables in TABEAM

    def unique_names(self) -> list:
        """Atom types in order of first appearance (sites%unique_atom, ffield.F90:613-633)."""
        seen = []
        for m in self.molecules:
            for s in m.sites:
                if s.name not in seen:
                    seen.append(s.name)
        return seen


_UNSUPPORTED_MOL = ("shell", "bond", "angl", "dihe", "inve", "rigi", "teth", "pmf")
_UNSUPPORTED_TOP = ("tbp", "fbp", "tersoff", "extern", "multi", "neut")


def write_field(path, fld: Field) -> None:
    """FIELD records: title, 'units', 'molecules n', per molecule type its name,
    'nummols', 'atoms' (runs of identical sites use the repeat count), 'constraints',
    'finish'; then 'vdw n' and 'close'.  Reals are written with all the digits of
    the double so that a FIELD read back gives the same parameters."""
    out = [fld.title[:80], f"units {fld.units}", f"molecules {len(fld.molecules)}"]
    for m in fld.molecules:
        out.append(m.name)
        out.append(f"nummols {m.nummols}")
        out.append(f"atoms {len(m.sites)}")
        k = 0
        while k < len(m.sites):
            s = m.sites[k]
            r = 1
            while k + r < len(m.sites) and m.sites[k + r] == s:
                r += 1
            out.append(f"{s.name:<8s} {s.mass!r:>20s} {s.charge!r:>22s} {r:6d} {s.freeze:2d}")
            k += r
        if m.constraints:
            out.append(f"constraints {len(m.constraints)}")
            for i, j, d in m.constraints:
                out.append(f"{i:6d} {j:6d} {float(d)!r:>22s}")
        out.append("finish")
    if fld.vdw:
        out.append(f"vdw {len(fld.vdw)}")
        for a, b, kind, prm in fld.vdw:
            out.append(f"{a:<8s} {b:<8s} {kind:<4s} " + " ".join(f"{float(p)!r:>22s}" for p in prm))
    if fld.metal:
        out.append(f"metal {len(fld.metal)}")
        for a, b, kind in fld.metal:
            out.append(f"{a:<8s} {b:<8s} {kind}")
    out.append("close")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def read_field(path) -> Field:
    """Reader for the FIELD directives of the path (keywords matched on their leading
    letters, case-insensitive, as ffield.F90 matches them)."""
    rec = _records(path)
    pos = [0]

    def next_words():
        while pos[0] < len(rec):
            line = rec[pos[0]]
            pos[0] += 1
            w = line.split()
            if w and not w[0].startswith("#"):
                return line, w
        raise ValueError(f"{path}: unexpected end of FIELD")

    title = rec[0].strip() if rec else ""
    pos[0] = 1
    units = None
    mols, vdw, metal = [], [], []
    while True:
        line, w = next_words()
        key = w[0].lower()
        if key.startswith("units"):
            u = w[1].lower() if len(w) > 1 else "internal"
            for name in ("ev", "kcal", "kj", "internal"):
                if u.startswith(name):
                    units = name
                    break
            else:
                if u.startswith("k"):
                    units = "k"
                else:
                    raise ValueError(f"{path}: energy unit '{u}' not recognised")
        elif key.startswith("molecul"):
            if units is None:
                raise ValueError(f"{path}: 'units' must precede 'molecules'")
            rest = [x for x in w[1:] if not x.lower().startswith("type")]
            for _ in range(int(to_real(rest[0]))):
                mols.append(_read_molecule(path, next_words))
        elif key.startswith("vdw"):
            if not mols:
                raise ValueError(f"{path}: 'vdw' before 'molecules'")
            for _ in range(int(to_real(w[1]))):
                _, v = next_words()
                kind = v[2].lower()
                if kind != "lj":
                    raise NotImplementedError(f"vdW form '{v[2]}': only 'lj' runs on this path")
                vdw.append((v[0][:8], v[1][:8], "lj", (to_real(v[3]), to_real(v[4]))))
        elif key.startswith("met"):
            for _ in range(int(to_real(w[1]))):
                _, v = next_words()
                kind = v[2].lower()
                if not kind.startswith("eam"):
                    raise NotImplementedError(f"metal form '{v[2]}': only tabulated 'eam' runs on this path")
                metal.append((v[0][:8], v[1][:8], "eam"))
        elif key.startswith("close"):
            break
        elif key.startswith(_UNSUPPORTED_TOP):
            raise NotImplementedError(f"FIELD directive '{w[0]}' is outside this path")
        else:
            raise ValueError(f"{path}: unknown FIELD directive '{w[0]}'")
    return Field(title=title, units=units or "internal", molecules=mols, vdw=vdw, metal=metal)


def _read_molecule(path, next_words) -> MoleculeType:
    line, _ = next_words()
    name = line.strip()
    nummols, sites, cons = 0, [], []
    while True:
        _, w = next_words()
        key = w[0].lower()
        if key.startswith("nummol"):
            nummols = int(to_real(w[1]))
        elif key.startswith("atoms"):
            nsite = int(to_real(w[1]))
            while len(sites) < nsite:
                _, a = next_words()
                nrept = int(to_real(a[3])) if len(a) > 3 else 1     # name mass charge nrept ifrz
                ifrz = int(to_real(a[4])) if len(a) > 4 else 0
                s = Site(a[0][:8], abs(to_real(a[1])), to_real(a[2]), 1 if ifrz != 0 else 0)
                sites.extend([s] * max(1, nrept))
            if len(sites) != nsite:
                raise ValueError(f"{path}: repeat counts overrun 'atoms {nsite}'")
        elif key.startswith("constr"):
            n = w[-1]
            for _ in range(int(to_real(n))):
                _, c = next_words()
                i, j = int(to_real(c[0])), int(to_real(c[1]))
                if max(i, j) > len(sites) or min(i, j) < 1:
                    raise ValueError(f"{path}: wrong index for atom in constraint")
                cons.append((i, j, to_real(c[2])))
        elif key.startswith("finish"):
            return MoleculeType(name=name, nummols=nummols, sites=sites, constraints=cons)
        elif key.startswith(_UNSUPPORTED_MOL):
            n = int(to_real(w[-1])) if len(w) > 1 else 0
            if n:
                raise NotImplementedError(f"FIELD molecular directive '{w[0]}' is outside this path")
        else:
            raise ValueError(f"{path}: unknown molecular directive '{w[0]}'")


# --------------------------------------------------------------------------------------
# TABEAM (tabulated EAM: metal_table_read, metal.F90:1489-1925)
# --------------------------------------------------------------------------------------
_TABEAM_KINDS = {"pair": "pair", "dens": "dens", "dden": "dens", "embe": "embe", "demb": "embe"}


def write_tabeam(path, tables, names, title="tabulated EAM", units="ev") -> None:
    """TABEAM: a title record, the number of tables, then per table a header
    'keyword atom1 [atom2] ngrid start finish' (atom2 for 'pair' only) and its values,
    four per record; energies (pair, embedding) in the FIELD units."""
    eng = ENGUNIT[units]
    out = [title[:80], f"{len(tables)}"]
    for t in tables:
        a, b = (names[k - 1] for k in t["types"])
        v = np.asarray(t["values"], np.float64)
        if t["kind"] != "dens":
            v = v / eng
        head = f"{t['kind']} {a}" + (f" {b}" if t["kind"] == "pair" else "")
        out.append(f"{head} {v.size} {float(t['start'])!r} {float(t['finish'])!r}")
        for k in range(0, v.size, 4):
            out.append(" ".join(f"{x!r}" for x in v[k:k + 4].tolist()))
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def read_tabeam(path, names, units="ev"):
    """Tables of a TABEAM file as the dicts System.eam holds (energies converted to
    internal units by the FIELD energy unit, as metal_table_read applies engunit)."""
    rec = _records(path)
    eng = ENGUNIT[units]
    tix = {nm: k + 1 for k, nm in enumerate(names)}
    k = 1
    numpot = int(to_real(rec[k].split()[0]))
    k += 1
    tabs = []
    for _ in range(numpot):
        w = rec[k].split()
        k += 1
        kw = w[0].lower()[:4]
        if kw not in _TABEAM_KINDS:
            raise NotImplementedError(f"TABEAM table '{w[0]}': pair, dens and embe run on this path")
        kind = _TABEAM_KINDS[kw]
        a = w[1][:8]
        rest = w[2:]
        b = a
        if kind == "pair":
            b, rest = rest[0][:8], rest[1:]
        ngrid, start, finish = int(to_real(rest[0])), to_real(rest[1]), to_real(rest[2])
        vals = []
        while len(vals) < ngrid:
            vals += [to_real(x) for x in rec[k].split()]
            k += 1
        v = np.asarray(vals[:ngrid], np.float64)
        if kind != "dens":
            v = v * eng
        if a not in tix or b not in tix:
            continue                       # the reference skips tables of absent species
        tabs.append({"kind": kind, "types": (tix[a], tix[b]), "start": start, "finish": finish, "values": v})
    return tabs


# --------------------------------------------------------------------------------------
# CONTROL (new style) and the GB300 sidecar
# --------------------------------------------------------------------------------------
# key -> (data type, unit class); data types as control.F90 registers them
KEYS = {
    "title": ("string", None),
    "cutoff": ("float", "length"),
    "padding": ("float", "length"),
    "timestep": ("float", "time"),
    "time_run": ("float", "steps"),
    "time_equilibration": ("float", "steps"),
    "ensemble": ("option", None),
    "ensemble_method": ("option", None),
    "ensemble_thermostat_coupling": ("float", "time"),
    "ensemble_thermostat_friction": ("float", "invtime"),
    "random_seed": ("vector", None),
    "temperature": ("float", "temperature"),
    "restart": ("option", None),
    "coul_method": ("option", None),
    "coul_dielectric_constant": ("float", None),
    "spme_alpha": ("float", "invlength"),
    "spme_precision": ("float", None),
    "spme_kvec": ("vector", None),
    "spme_nsplines": ("int", None),
    "vdw_method": ("option", None),
    "vdw_cutoff": ("float", "length"),
    "shake_tolerance": ("float", "length"),
    "shake_max_iter": ("int", None),
    "print_frequency": ("float", "steps"),
    "stats_frequency": ("float", "steps"),
    "stack_size": ("float", "steps"),
    "data_dump_frequency": ("float", "steps"),
    "rdf_binsize": ("float", "length"),
    "io_file_config": ("string", None),
    "io_file_field": ("string", None),
    "io_file_statis": ("string", None),
    "io_file_revive": ("string", None),
    "io_file_revcon": ("string", None),
}
# Settings of the GPU forms.  The reference's CONTROL parser stops on unknown keys, so
# these live in a separate file (GBCONTROL) with the same syntax.
GB_KEYS = {
    "gb_precision": ("option", None),      # fp64 | mixed
    "gb_mts_k": ("int", None),
    "gb_mts_tol": ("float", None),
    "gb_mts_train": ("int", None),
    "gb_device": ("int", None),
}
_UNITS = {
    "length": {"": 1.0, "ang": 1.0, "angs": 1.0, "angstrom": 1.0, "internal_l": 1.0, "nm": 10.0,
               "bohr": 0.52917721092, "pm": 0.01},
    "invlength": {"": 1.0, "ang^-1": 1.0, "1/ang": 1.0, "internal_l^-1": 1.0, "nm^-1": 0.1},
    "time": {"": 1.0, "ps": 1.0, "internal_t": 1.0, "fs": 1.0e-3, "ns": 1.0e3},
    "invtime": {"": 1.0, "ps^-1": 1.0, "1/ps": 1.0, "internal_t^-1": 1.0, "fs^-1": 1.0e3, "ns^-1": 1.0e-3},
    "temperature": {"": 1.0, "k": 1.0},
    "steps": {"": 1.0, "steps": 1.0, "step": 1.0},
}
CONTROL_DEFAULTS = {
    "time_equilibration": 0, "ensemble": "nve", "temperature": 0.0, "restart": "clean",
    "coul_method": "off", "coul_dielectric_constant": 1.0, "spme_nsplines": 8,
    "vdw_method": "tabulated", "shake_tolerance": 1.0e-6, "shake_max_iter": 250,
    "print_frequency": 0, "stats_frequency": 0, "stack_size": 0, "data_dump_frequency": 1000,
    "rdf_binsize": 0.05, "padding": 0.0, "timestep": 0.0, "time_run": 0,
}


def _convert(key, val, unit, keys):
    kind, ucls = keys[key]
    if kind == "float":
        x = to_real(val)
        if ucls is not None:
            table = _UNITS[ucls]
            u = unit.lower()
            if u not in table:
                raise ValueError(f"unit '{unit}' not understood for '{key}'")
            x *= table[u]
            if ucls == "steps":
                return int(round(x))
        return x
    if kind == "int":
        return int(round(to_real(val)))
    return val


def read_control(path, keys=None) -> dict:
    """Parse new-style CONTROL: one 'key value [unit]' per line, '#' or '!' starts a
    comment, vectors in brackets (continued with '&'), a key may appear once, and the
    first key is 'title' (else the file is old-style, which is not read here).
    Values come back in internal units (A, ps, K, steps)."""
    keys = KEYS if keys is None else keys
    rec = _records(path)
    out = {}
    i = 0
    first = True
    while i < len(rec):
        line = rec[i]
        i += 1
        cut = min([p for p in (line.find("#"), line.find("!")) if p >= 0], default=-1)
        if cut >= 0:
            line = line[:cut]
        w = line.split()
        if not w:
            continue
        key = w[0].lower()
        if first and keys is KEYS and key != "title":
            raise ValueError(f"{path}: old-style CONTROL (first key is not 'title') is not read here")
        first = False
        if key not in keys:
            raise ValueError(f"{path}: Unrecognised key {key}")
        if key in out:
            raise ValueError(f"{path}: Param {key} already set")
        kind = keys[key][0]
        rest = line.split(None, 1)[1] if len(w) > 1 else ""
        if kind == "string":
            out[key] = rest.strip()
        elif kind == "vector":
            while "&" in rest:
                rest = rest[:rest.index("&")] + " " + rec[i]
                i += 1
            rest = rest.strip()
            if not rest.startswith("["):
                raise ValueError(f"{path}: vector value of '{key}' needs brackets")
            j = rest.rindex("]")
            out[key] = [to_real(x) for x in rest[1:j].split()]
        elif kind == "option":
            if not rest.strip():
                raise ValueError(f"{path}: Missing option for {key}")
            out[key] = rest.split()[0].lower()
        else:
            parts = rest.split()
            if not parts:
                raise ValueError(f"{path}: missing value for {key}")
            if kind == "int" and len(parts) > 1:
                raise ValueError(f"{path}: Unexpected junk {' '.join(parts[1:])} after key {key}")
            if len(parts) > 2:
                raise ValueError(f"{path}: Unexpected junk {' '.join(parts[2:])} after key {key}")
            out[key] = _convert(key, parts[0], parts[1] if len(parts) > 1 else "", keys)
    return out


_WRITE_UNITS = {"length": "ang", "invlength": "ang^-1", "time": "ps", "invtime": "ps^-1", "temperature": "K",
                "steps": "steps"}


def write_control(path, values: dict, keys=None) -> None:
    """Write 'key value [unit]' lines, 'title' first, values in internal units."""
    keys = KEYS if keys is None else keys
    order = (["title"] if "title" in values else []) + [k for k in values if k != "title"]
    out = []
    for k in order:
        if k not in keys:
            raise ValueError(f"unknown key {k}")
        kind, ucls = keys[k]
        v = values[k]
        if kind == "vector":
            out.append(f"{k} [" + " ".join(str(int(x)) if float(x).is_integer() else repr(float(x))
                                         for x in v) + "]")
        elif kind == "float":
            unit = _WRITE_UNITS.get(ucls, "")
            s = str(int(v)) if ucls == "steps" else repr(float(v))
            out.append(f"{k} {s} {unit}".rstrip())
        else:
            out.append(f"{k} {v}")
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


# --------------------------------------------------------------------------------------
# System <-> files
# --------------------------------------------------------------------------------------
def _molecule_of(s: System):
    """Atoms of each molecule: connected components of the constraint graph, in
    order, with singletons for unconstrained atoms.  Molecules must be contiguous."""
    n = s.natms
    parent = np.arange(n)

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    lc = s.listcon.reshape(-1, 3) if s.ntcons else np.zeros((0, 3), np.int64)
    for _, gi, gj in lc:
        a, b = find(gi - 1), find(gj - 1)
        if a != b:
            parent[max(a, b)] = min(a, b)
    roots = np.array([find(a) for a in range(n)])
    starts = np.flatnonzero(np.r_[True, roots[1:] != roots[:-1]])
    ends = np.r_[starts[1:], n]
    for a0, a1 in zip(starts, ends):
        if np.any(roots[a0:a1] != a0):
            raise ValueError("a constrained molecule is not contiguous in atom order")
    return list(zip(starts.tolist(), ends.tolist())), lc


def field_from_system(s: System, units: str | None = None, title: str | None = None):
    """FIELD description of a System and the atom order it implies.

    Returns (Field, perm): perm[k] is the System atom written as the k-th CONFIG
    atom.  Molecules with the same sites and constraints form one molecule type;
    types are listed in order of first appearance and their molecules written
    together, as FIELD requires (one block of nummols molecules per type)."""
    if units is None:
        units = "ev" if s.eam else "kj"
    names = list(s.type_names) or [f"T{k + 1}" for k in range(s.ntypes)]
    mols, lc = _molecule_of(s)
    prm = s.prmcon
    cons_of = {}
    for kind, gi, gj in lc:
        cons_of.setdefault(gi - 1, []).append((int(gi) - 1, int(gj) - 1, float(prm[kind - 1])))
    sigs, members = [], {}
    for a0, a1 in mols:
        sites = tuple((names[s.ltype[a] - 1], float(s.weight[a]), float(s.chge[a]), int(s.lfrzn[a] != 0))
                      for a in range(a0, a1))
        cons = []
        for a in range(a0, a1):
            for gi, gj, d in cons_of.get(a, []):
                cons.append((gi - a0 + 1, gj - a0 + 1, d))
        key = (sites, tuple(cons))
        if key not in members:
            sigs.append(key)
            members[key] = []
        members[key].append((a0, a1))
    mtypes, perm = [], []
    for key in sigs:
        sites, cons = key
        nm = sites[0][0] if len(sites) == 1 else "-".join(x[0] for x in sites)
        mtypes.append(MoleculeType(name=nm, nummols=len(members[key]),
                                   sites=[Site(*x) for x in sites], constraints=list(cons)))
        for a0, a1 in members[key]:
            perm.extend(range(a0, a1))
    eng = ENGUNIT[units]
    vdw = []
    nt = s.ntypes
    for a in range(1, nt + 1):
        for b in range(1, a + 1):
            k = a * (a - 1) // 2 + b - 1
            kind, eps, sig = s.vdw_prm[3 * k:3 * k + 3]
            if int(kind) == 1:
                vdw.append((names[b - 1], names[a - 1], "lj", (eps / eng, sig)))
    metal = []
    if s.eam:
        lst = s.metal_listed if s.metal_listed is not None else np.ones(nt * (nt + 1) // 2, np.int32)
        for a in range(1, nt + 1):
            for b in range(1, a + 1):
                if lst[a * (a - 1) // 2 + b - 1]:
                    metal.append((names[a - 1], names[b - 1], "eam"))
    fld = Field(title=title or s.name, units=units, molecules=mtypes, vdw=vdw, metal=metal)
    return fld, np.asarray(perm, np.int64)


def control_from_system(s: System, steps: int, temperature: float, stats_every: int = 1) -> dict:
    """New-style CONTROL values that select the same path and parameters as the System."""
    return {
        "title": s.name,
        "cutoff": s.rcut, "padding": s.rpad, "vdw_cutoff": s.rcut,
        "timestep": s.tstep, "time_run": int(steps), "time_equilibration": 0,
        "ensemble": "nve", "temperature": float(temperature),
        "restart": "noscale",                      # keep the CONFIG velocities as written
        "coul_method": "spme" if np.any(s.chge != 0.0) else "off", "coul_dielectric_constant": s.epsq,
        "spme_alpha": s.alpha, "spme_kvec": [int(k) for k in s.kmax], "spme_nsplines": s.nsplines,
        "vdw_method": "direct" if s.vdw_direct else "tabulated",
        "shake_tolerance": s.shake_tol, "shake_max_iter": s.shake_maxit,
        "stats_frequency": int(stats_every), "print_frequency": int(stats_every),
    }


def config_from_system(s: System, perm=None, levcfg: int = 1, frc=None, step: int = 0,
                       time: float = 0.0) -> Config:
    perm = np.arange(s.natms) if perm is None else np.asarray(perm)
    names = list(s.type_names) or [f"T{k + 1}" for k in range(s.ntypes)]
    pos = np.stack([s.x, s.y, s.z], 1)[perm]
    vel = np.stack([s.vx, s.vy, s.vz], 1)[perm]
    return Config(title=s.name, levcfg=levcfg, imcon=1 if _is_cubic(s.cell) else 3, cell=s.cell.copy(),
                  names=[names[t - 1] for t in s.ltype[perm]], index=np.arange(1, s.natms + 1),
                  pos=pos, vel=vel if levcfg >= 1 else None,
                  frc=(np.asarray(frc)[perm] if frc is not None else None),
                  step=step, tstep=s.tstep, time=time)


def _is_cubic(cell) -> bool:
    c = np.asarray(cell).reshape(3, 3)
    return bool(np.all(c == np.diag(np.diag(c))) and c[0, 0] == c[1, 1] == c[2, 2])


def spme_kvec_from_precision(precision: float, rcut: float, cell) -> tuple:
    """alpha and K from 'spme_precision' (control.F90:1705-1711)."""
    precision = max(min(precision, 0.5), 1.0e-20)
    alpha = ewald_alpha(precision, rcut)
    tol = math.sqrt(abs(math.log(precision * rcut)))
    tol1 = math.sqrt(-math.log(precision * rcut * (2.0 * tol * alpha) ** 2))
    widths = _widths(cell)
    return alpha, tuple(2 * int(round(0.25 + w * alpha * tol1 / math.pi)) for w in widths)


def _widths(cell):
    """Perpendicular widths of the cell (dcell's celprp(7:9))."""
    c = np.asarray(cell, np.float64).reshape(3, 3)
    vol = abs(np.linalg.det(c))
    a, b, cc = c
    return (vol / np.linalg.norm(np.cross(b, cc)), vol / np.linalg.norm(np.cross(cc, a)),
            vol / np.linalg.norm(np.cross(a, b)))


def system_from_files(cfg: Config, fld: Field, ctl: dict, tabeam=None) -> System:
    """Build a System from CONFIG, FIELD and CONTROL (and the TABEAM file, path or
    tables, when FIELD lists 'eam' metal potentials).  Atom i of the System is atom
    i of the CONFIG; FIELD molecule types assign sites to atoms in the same order."""
    c = dict(CONTROL_DEFAULTS)
    c.update(ctl)
    ensemble_from_control(c)                       # refuses ensembles outside the path
    if c["coul_method"] not in ("spme", "off"):
        raise NotImplementedError(f"coul_method '{c['coul_method']}': spme (or off, uncharged) runs here")
    if "cutoff" not in c:
        raise ValueError("CONTROL needs 'cutoff'")
    rcut = float(c["cutoff"])
    if "vdw_cutoff" in c and c["vdw_cutoff"] > 0 and abs(c["vdw_cutoff"] - rcut) > 1e-12:
        raise NotImplementedError("vdw_cutoff different from cutoff is not run on this path")
    if cfg.imcon not in (1, 2, 3):
        raise NotImplementedError(f"imcon {cfg.imcon}: this path runs periodic boxes (1, 2, 3)")
    names = fld.unique_names()
    tix = {nm: k + 1 for k, nm in enumerate(names)}
    ltype, chge, weight, frz, listcon, prmcon, excl = [], [], [], [], [], [], {}
    base = 0
    for m in fld.molecules:
        ptypes = []
        for i, j, d in m.constraints:
            prmcon.append(d)
            ptypes.append(len(prmcon))
        for _ in range(m.nummols):
            for st in m.sites:
                ltype.append(tix[st.name])
                chge.append(st.charge)
                weight.append(st.mass)
                frz.append(st.freeze)
            for (i, j, _d), t in zip(m.constraints, ptypes):
                gi, gj = base + i, base + j
                listcon += [t, gi, gj]
                excl.setdefault(gi, set()).add(gj)
                excl.setdefault(gj, set()).add(gi)
            base += len(m.sites)
    n = len(ltype)
    if n != cfg.natms:
        raise ValueError(f"FIELD describes {n} atoms, CONFIG holds {cfg.natms}")
    cfg_names = [x[:8] for x in cfg.names]
    want = [names[t - 1] for t in ltype]
    if cfg_names != want:
        bad = next(k for k in range(n) if cfg_names[k] != want[k])
        raise ValueError(f"CONFIG atom {bad + 1} is '{cfg_names[bad]}', FIELD says '{want[bad]}'")
    nt = len(names)
    eng = ENGUNIT[fld.units]
    if c["coul_method"] == "off" and any(q != 0.0 for q in chge):
        raise NotImplementedError("charged sites with coul_method off are not run on this path")
    eam, listed = None, None
    if fld.metal:
        listed = np.zeros(nt * (nt + 1) // 2, np.int32)
        for a_nm, b_nm, _kind in fld.metal:
            a, b = max(tix[a_nm], tix[b_nm]), min(tix[a_nm], tix[b_nm])
            listed[a * (a - 1) // 2 + b - 1] = 1
        if tabeam is None:
            raise ValueError("FIELD lists eam metal potentials: a TABEAM file is needed")
        eam = read_tabeam(tabeam, names, fld.units) if isinstance(tabeam, (str, bytes)) or hasattr(tabeam, "__fspath__") else tabeam
    vdw_prm = np.zeros(3 * (nt * (nt + 1) // 2))
    for a_nm, b_nm, kind, prm in fld.vdw:
        a, b = tix[a_nm], tix[b_nm]
        if a < b:
            a, b = b, a
        k = a * (a - 1) // 2 + b - 1
        vdw_prm[3 * k:3 * k + 3] = (1.0, prm[0] * eng, prm[1])
    maxex = max((len(v) for v in excl.values()), default=0)
    list_excl = None
    if maxex:
        list_excl = np.zeros((n, maxex + 1), np.int32)
        for gi, js in excl.items():
            js = sorted(js)
            list_excl[gi - 1, 0] = len(js)
            list_excl[gi - 1, 1:1 + len(js)] = js
    if "spme_alpha" in c and "spme_precision" in c:
        raise ValueError("Cannot specify both precision and manual spme parameters")
    if c["coul_method"] == "off":                  # no reciprocal space: grid parameters unused
        alpha, kmax = float(c.get("spme_alpha", 0.3)), tuple(int(x) for x in c.get("spme_kvec", (16, 16, 16)))
    elif "spme_alpha" in c:
        alpha = float(c["spme_alpha"])
        if "spme_kvec" not in c:
            raise ValueError("CONTROL with spme_alpha needs spme_kvec")
        kmax = tuple(int(x) for x in c["spme_kvec"])
    else:
        alpha, kmax = spme_kvec_from_precision(float(c.get("spme_precision", 1.0e-6)), rcut, cfg.cell)
    nspl = int(c["spme_nsplines"])                 # control.F90:1652-1675: at least 3, even
    nspl = max(nspl, 3)
    nspl += nspl % 2
    vel = cfg.vel if cfg.vel is not None else np.zeros((n, 3))
    return System(
        name=cfg.title or fld.title, cell=np.asarray(cfg.cell, np.float64).copy(),
        ltype=np.asarray(ltype, np.int32), chge=np.asarray(chge, np.float64),
        weight=np.asarray(weight, np.float64), lfrzn=np.asarray(frz, np.int32), vdw_prm=vdw_prm,
        x=cfg.pos[:, 0].copy(), y=cfg.pos[:, 1].copy(), z=cfg.pos[:, 2].copy(),
        vx=vel[:, 0].copy(), vy=vel[:, 1].copy(), vz=vel[:, 2].copy(),
        rcut=rcut, rpad=float(c["padding"]), alpha=alpha, kmax=kmax, ntypes=nt, nsplines=nspl,
        tstep=float(c["timestep"]), shake_tol=float(c["shake_tolerance"]),
        listcon=np.asarray(listcon, np.int32), prmcon=np.asarray(prmcon, np.float64),
        max_exclude=maxex, list_excl=list_excl, vdw_direct=1 if c["vdw_method"] == "direct" else 0,
        type_names=tuple(names), epsq=float(c["coul_dielectric_constant"]),
        shake_maxit=int(c["shake_max_iter"]), eam=eam, metal_listed=listed)


_NVT_METHODS = {"berendsen": "berendsen", "hoover": "nose-hoover", "nose": "nose-hoover",
                "nose-hoover": "nose-hoover", "langevin": "langevin"}


def ensemble_from_control(ctl: dict) -> dict:
    """Ensemble of the VV stages from CONTROL, as control.F90:570-640 selects it:
    'ensemble nve', or 'ensemble nvt' with 'ensemble_method' berendsen / hoover
    (tau_t from ensemble_thermostat_coupling) or langevin (chi from
    ensemble_thermostat_friction), at 'temperature', with 'random_seed' shifts."""
    ens = str(ctl.get("ensemble", "nve")).lower()
    if ens in ("nve", "pmf"):
        return {"kind": "nve"}
    if ens != "nvt":
        raise NotImplementedError(f"ensemble '{ens}': nve and nvt run on this path")
    method = str(ctl.get("ensemble_method", "")).lower()
    if method not in _NVT_METHODS:
        raise NotImplementedError(f"nvt ensemble_method '{method}': berendsen, hoover and langevin run here")
    kind = _NVT_METHODS[method]
    out = {"kind": kind, "temp": float(ctl.get("temperature", 0.0)),
           "tau_t": float(ctl.get("ensemble_thermostat_coupling", 0.0)),
           "chi": float(ctl.get("ensemble_thermostat_friction", 0.0))}
    if "random_seed" in ctl:
        out["seed"] = tuple(int(round(x)) for x in ctl["random_seed"][:3])
    if kind == "langevin" and "ensemble_thermostat_friction" not in ctl:
        raise ValueError("nvt langevin needs ensemble_thermostat_friction")
    return out


def emit_inputs(s: System, directory, steps: int, temperature: float, stats_every: int = 1,
                gb: dict | None = None):
    """Write CONFIG, FIELD, CONTROL (and GBCONTROL when gb settings are given) for a
    System, plus the raw arrays in 'arrays.npz' in System order.  Returns perm."""
    import os
    os.makedirs(directory, exist_ok=True)
    fld, perm = field_from_system(s)
    write_field(os.path.join(directory, "FIELD"), fld)
    write_config(os.path.join(directory, "CONFIG"), config_from_system(s, perm, levcfg=1))
    write_control(os.path.join(directory, "CONTROL"), control_from_system(s, steps, temperature, stats_every))
    if gb:
        write_control(os.path.join(directory, "GBCONTROL"), gb, GB_KEYS)
    if s.eam:
        write_tabeam(os.path.join(directory, "TABEAM"), s.eam, list(s.type_names), title=s.name,
                     units=fld.units)
    np.savez(os.path.join(directory, "arrays.npz"), cell=s.cell, ltype=s.ltype, chge=s.chge,
             weight=s.weight, lfrzn=s.lfrzn, vdw_prm=s.vdw_prm, x=s.x, y=s.y, z=s.z, vx=s.vx,
             vy=s.vy, vz=s.vz, listcon=s.listcon, prmcon=s.prmcon,
             list_excl=s.list_excl if s.list_excl is not None else np.zeros((0, 1), np.int32),
             perm=perm, rcut=s.rcut, rpad=s.rpad, alpha=s.alpha, kmax=np.asarray(s.kmax),
             nsplines=s.nsplines, tstep=s.tstep, shake_tol=s.shake_tol)
    return perm


# --------------------------------------------------------------------------------------
# Long-range vdW correction (added to the short-range energy and virial in STATIS)
# --------------------------------------------------------------------------------------
def vdw_long_range(s: System) -> tuple:
    """(elrc, vlrc) for 12-6 LJ pairs beyond the cutoff (vdw.F90:617-967):
    elrc = 2 pi / V * sum_{a>=b} c_ab (N_a N_b - F_a F_b) * 4 eps (s^12/(9 r^9) - s^6/(3 r^3)),
    plrc likewise with 8 eps (6 s^12/(9 r^9) - s^6/r^3) / 3, vlrc = -3 V plrc; c_ab = 2 for
    a /= b.  N are atoms per type and F frozen atoms per type."""
    vol = s.volume()
    nt = s.ntypes
    num = np.bincount(s.ltype, minlength=nt + 1)[1:].astype(np.float64)
    nfz = np.bincount(s.ltype[s.lfrzn != 0], minlength=nt + 1)[1:].astype(np.float64)
    r = s.rcut
    elrc = plrc = 0.0
    for a in range(1, nt + 1):
        for b in range(1, a + 1):
            k = a * (a - 1) // 2 + b - 1
            kind, eps, sig = s.vdw_prm[3 * k:3 * k + 3]
            if int(kind) != 1:
                continue
            eadd = 4.0 * eps * (sig ** 12 / (9.0 * r ** 9) - sig ** 6 / (3.0 * r ** 3))
            padd = 8.0 * eps * (6.0 * sig ** 12 / (9.0 * r ** 9) - sig ** 6 / r ** 3)
            if a != b:
                eadd *= 2.0
                padd *= 2.0
            den = 2.0 * math.pi * (num[a - 1] * num[b - 1] - nfz[a - 1] * nfz[b - 1]) / vol ** 2
            elrc += vol * den * eadd
            plrc += den * padd / 3.0
    return elrc, plrc * (-3.0 * vol)


# --------------------------------------------------------------------------------------
# STATIS and REVIVE
# --------------------------------------------------------------------------------------
def _cell_angles(cell):
    c = np.asarray(cell, np.float64).reshape(3, 3)
    a, b, cc = c
    ang = lambda u, v: math.degrees(math.acos(float(np.dot(u, v) / (np.linalg.norm(u) * np.linalg.norm(v)))))
    return ang(b, cc), ang(a, cc), ang(a, b)          # alpha, beta, gamma


class Statistics:
    """Per-step observables and their accumulators, kept as statistics_collect keeps them.

    stpval has indices 0..mxnstk with mxnstk = 51 + ntypes (bounds.F90:1002); the stack
    holds max(100, stack_size) samples (bounds.F90:996)."""

    def __init__(self, s: System, units: str = "kj", stack_size: int = 0, nsteql: int = 0):
        self.sys = s
        self.units = units
        self.engunit = ENGUNIT[units]
        self.ntypes = s.ntypes
        self.mxnstk = 51 + s.ntypes
        self.mxstak = max(100, int(stack_size))
        self.nsteql = nsteql
        n = self.mxnstk + 1
        self.stpval = np.zeros(n)
        self.stpvl0 = np.zeros(n)
        self.sumval = np.zeros(n)
        self.ssqval = np.zeros(n)
        self.zumval = np.zeros(n)
        self.ravval = np.zeros(n)
        self.stkval = np.zeros((self.mxstak, n))
        self.numacc = 0
        self.iadd = 36 + s.ntypes
        self.degfre = 3 * int(np.sum(s.lfrzn == 0)) - 3 - s.ntcons     # temperature.F90:109-143
        self.elrc, self.vlrc = vdw_long_range(s)
        nf = np.bincount(s.ltype[s.lfrzn == 0], minlength=s.ntypes + 1)[1:]
        self.num_type_nf = nf.astype(np.float64)

    def header(self, title: str) -> str:
        """The two header records of a fresh STATIS (statistics.F90:1011-1025)."""
        return f"title: '{title}'\nenergy unitS: {STATIS_UNITS[self.units]}\n"

    def collect(self, nstep: int, st: dict, cell, amsd=None) -> None:
        """Fill stpval for one step from the path's step scalars (gb_step_stats fields)
        and update the running sums; st['stress'] etc. are 9-vectors."""
        eu = self.engunit
        vol = abs(float(np.linalg.det(np.asarray(cell).reshape(3, 3))))
        engcpe = st["engcpe_rc"] + st["engcpe_rl"] + st["engcpe_ex"]
        vircpe = st["vircpe_rc"] + st["vircpe_rl"] + st["vircpe_ex"]
        # two_body.F90:780-781: short range = metal (pair + embedding) + vdW + long-range vdW
        engsrp = st.get("engmet", 0.0) + st["engvdw"] + self.elrc
        virsrp = st.get("virmet", 0.0) + st["virvdw"] + self.vlrc
        engke = st["engke"]
        vircon = st["vircon"]
        stpcfg = engcpe + engsrp
        stpeng = stpcfg + engke
        stptmp = 2.0 * engke / (BOLTZ * self.degfre)
        virtot = vircpe + virsrp
        stpvir = virtot + vircon
        stpprs = (2.0 * engke - stpvir) / (3.0 * vol)
        stpeth = stpeng + stpprs * vol
        stress = np.asarray(st["stress"], np.float64).copy()
        stress[[0, 4, 8]] += -self.vlrc / 3.0                # two_body.F90:787-790
        strtot = np.asarray(st.get("strcon", np.zeros(9))) + stress + np.asarray(st["strkin"])
        al, be, ga = _cell_angles(cell)
        v = self.stpval
        v[:] = 0.0
        consv = float(st.get("consv", 0.0))              # thermostat's conserved-energy term
        v[0] = consv / eu
        v[1] = (stpeng + consv) / eu
        v[2] = stptmp
        v[3] = stpcfg / eu
        v[4] = engsrp / eu
        v[5] = engcpe / eu
        v[10] = stpeth / eu
        v[12] = stpvir / eu
        v[13] = virsrp / eu
        v[14] = vircpe / eu
        v[17] = vircon / eu
        v[19] = vol
        v[23], v[24], v[25] = al, be, ga
        v[27] = stpprs * PRSUNT
        v[28:37] = strtot * PRSUNT / vol
        if amsd is not None:
            nf = self.num_type_nf
            v[37:37 + self.ntypes] = np.where(nf > 0, np.asarray(amsd) / np.maximum(nf, 1), 0.0)
        if nstep == 0:
            return
        kst = (nstep - 1) % self.mxstak
        if nstep > self.mxstak:
            self.zumval -= self.stkval[kst]
        self.stkval[kst] = v
        self.zumval += v
        self.ravval = self.zumval / float(min(self.mxstak, nstep))
        if nstep > self.nsteql:
            self.numacc += 1
            s2 = 1.0 / self.numacc
            s1 = (self.numacc - 1) / self.numacc
            if nstep == self.nsteql + 1:
                self.stpvl0 = v.copy()
            d = v - self.stpvl0
            self.ssqval = s1 * (self.ssqval + s2 * (d - self.sumval) ** 2)
            self.sumval = s1 * self.sumval + s2 * d

    def statis_record(self, nstep: int, time: float) -> str:
        """One STATIS record (statistics.F90:1345-1346): nstep (i10), time (1p,e14.6),
        the count (i10), then stpval(1:27), stpval(0), stpval(28:iadd), five per line
        in (1p,5e14.6)."""
        v = self.stpval
        vals = list(v[1:28]) + [v[0]] + list(v[28:self.iadd + 1])
        out = [fmt_i(nstep, 10) + fmt_e(time, 14, 6, 1) + fmt_i(len(vals), 10)]
        for k in range(0, len(vals), 5):
            out.append("".join(fmt_e(float(x), 14, 6, 1) for x in vals[k:k + 5]))
        return "\n".join(out) + "\n"

    # REVIVE, unformatted branch of system_revive: records of reals, each framed by
    # 4-byte little-endian lengths as gfortran writes sequential unformatted files.
    def write_revive(self, path, rcut: float, megatm: int, nstep: int, tstep: float, time: float,
                     tmst: float, strcon, stress, rbin: float = 0.05, chi_t: float = 0.0,
                     cint: float = 0.0) -> None:
        recs = [np.array([rcut, rbin, float(megatm)]),
                np.array([float(nstep), tstep, time, tmst, float(self.numacc), chi_t, 0.0, cint]),
                np.zeros(9),                              # thermo%eta
                self.stpval, self.stpvl0, self.sumval, self.ssqval, self.zumval, self.ravval,
                self.stkval.T.reshape(-1),                # stkval(1:mxstak, 0:mxnstk), column-major
                np.asarray(strcon, np.float64), np.zeros(9), np.asarray(stress, np.float64)]
        with open(path, "wb") as fh:
            for r in recs:
                b = np.ascontiguousarray(r, "<f8").tobytes()
                fh.write(struct.pack("<i", len(b)) + b + struct.pack("<i", len(b)))

    def read_revive(self, path) -> dict:
        """Read a REVIVE written by write_revive back into the accumulators."""
        recs = []
        with open(path, "rb") as fh:
            data = fh.read()
        p = 0
        while p < len(data):
            (n,) = struct.unpack_from("<i", data, p)
            recs.append(np.frombuffer(data, "<f8", n // 8, p + 4).copy())
            (m,) = struct.unpack_from("<i", data, p + 4 + n)
            if m != n:
                raise ValueError(f"{path}: record markers disagree ({n} vs {m})")
            p += n + 8
        n = self.mxnstk + 1
        if len(recs) < 13 or recs[3].size != n or recs[9].size != n * self.mxstak:
            raise ValueError(f"{path}: REVIVE layout does not match this system's statistics sizes")
        (self.stpval, self.stpvl0, self.sumval, self.ssqval, self.zumval, self.ravval) = recs[3:9]
        self.stkval = recs[9].reshape(n, self.mxstak).T.copy()
        self.numacc = int(recs[1][4])
        return {"rcut": recs[0][0], "rbin": recs[0][1], "megatm": int(recs[0][2]),
                "nstep": int(recs[1][0]), "tstep": recs[1][1], "time": recs[1][2], "tmst": recs[1][3],
                "chi_t": recs[1][5], "cint": recs[1][7],
                "strcon": recs[10], "strpmf": recs[11], "stress": recs[12]}
