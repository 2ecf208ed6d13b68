"""NVT thermostats of the oracle (CPU): the random stream of the Langevin forces
against an independent Python restatement of sarurnd / box_mueller_saru3
(numerics.F90:458-635, :745-803), and physical properties of the Berendsen,
Nose-Hoover and Langevin stages (nvt_berendsen.F90, nvt_nose_hoover.F90,
nvt_langevin.F90).  The GPU stages are compared with these in
test_gpu_thermostats.py."""
import math

import numpy as np
import pytest

from dlpoly_gb300 import systems

BOLTZ = 0.831451115
M64 = (1 << 64) - 1
T32 = 1 << 32


def _u64(x):
    return x & M64


def _shl(x, n):            # Ishft(x, n), n > 0, on a 64-bit integer
    v = _u64(_u64(x) << n)
    return v - (1 << 64) if v >> 63 else v


def _shr(x, n):            # Ishft(x, -n): logical right shift of the 64-bit pattern
    return _u64(x) >> n


def _int32(x):             # Int(Int(x), Kind=li): low 32 bits, sign-extended
    v = x & 0xFFFFFFFF
    return v - T32 if v >> 31 else v


def _fmod(x, y):           # Fortran Mod: sign of the dividend
    r = abs(x) % y
    return -r if x < 0 else r


def _prod(a, b):           # Int(Mod(a*b in double, 2^32), Kind=li)
    return int(math.fmod(float(a) * float(b), 4294967296.0))


def saru_py(a, b, c):
    s1, s2, s3 = (_fmod(v, T32) for v in (a, b, c))
    s1, s2, s3 = (v + T32 if v < 0 else v for v in (s1, s2, s3))
    s3 = _fmod(s3 ^ (_shl(s1, 7) ^ _shr(s2, 6)), T32)
    s2 = _fmod(s2 + (_shr(s1, 4) ^ _shr(s3, 15)), T32)
    s1 = _fmod(s1 ^ (_shl(s2, 9) + _shl(s3, 8)), T32)
    s3 = _fmod(s3 ^ _prod(2771807053.0, _shr(s2, 11) ^ _shl(s1, 1)), T32)
    s2 = _fmod(s2 + _prod(1925059961.0, _shl(s1, 4) ^ _shr(s3, 16)), T32)
    t = _prod(1060677357.0, _shr(s3, 5) ^ _shr(_int32(s2), 22))
    t = t + T32 if t < 0 else t
    s1 = _fmod(s1 ^ t, T32)
    s2 = _fmod(s2 + _prod(s1, s3), T32)
    s1 = _fmod(s1 + (s3 ^ _shr(s2, 2)), T32)
    s2 = s2 ^ _shr(_int32(s2), 17)
    state = _prod(2044649123.0, s1 ^ _shr(_int32(s1), 14))
    wstate = _fmod((state + s2) ^ _shr(_int32(state), 8), T32)
    state = _fmod(state + _prod(wstate, wstate ^ 3722418165), T32)
    wstate = _fmod(2882246391 + _shr(wstate, 1), T32)
    state = _fmod(_prod(1273716057.0, state) + 637592055, T32)
    wstate = _fmod(wstate + 2148127051 + (_shr(_int32(wstate), 31) & 3666320093), T32)
    v = _fmod((state ^ _shr(state, 26)) + wstate, T32)
    u32 = _prod(v ^ _shr(v, 20), 1767372199.0)
    r32 = 2.0 ** -32
    return (float(_int32(u32)) * r32 + (0.5 + 0.5 * r32)) + float(state) * (r32 * r32)


def gauss3_py(i, j, k=0):
    out = []
    for want in (2, 1):
        r0 = 1.0
        while r0 <= 2.2250738585072014e-308 or r0 >= 1.0:
            r1 = 2.0 * saru_py(i, j, k) - 1.0
            r2 = 2.0 * saru_py(i, j, k + 1) - 1.0
            r0 = r1 * r1 + r2 * r2
            k += 2
        r0 = math.sqrt(-2.0 * math.log(r0) / r0)
        out += [r0 * r1, r0 * r2][:want]
    return out


def _seeds(n, seed=11):
    rng = np.random.default_rng(seed)
    a = rng.integers(1, 300000, n)
    b = rng.integers(-20000, 20000, n)
    c = rng.integers(0, 8, n)
    a[:4] = [1, 2**31 - 1, 2**31, 4294967295]     # values that cross the signed 32-bit range
    b[:4] = [0, -1, 2**31, -(2**31)]
    return a, b, c


def test_saru_stream_matches_python_restatement(oracle_lib):
    a, b, c = _seeds(3000)
    got = oracle_lib.rng_eval(0, a, b, c)
    want = np.array([saru_py(int(x), int(y), int(z)) for x, y, z in zip(a, b, c)])
    assert np.array_equal(got, want)
    assert np.all((got > 0.0) & (got < 1.0))


def test_gaussians_match_and_are_unit_normal(oracle_lib):
    a, b, c = _seeds(400, seed=5)
    c[:] = 0
    got = oracle_lib.rng_eval(1, a, b, c)
    want = np.array([gauss3_py(int(x), int(y)) for x, y in zip(a, b)])
    assert np.array_equal(got, want)
    big = oracle_lib.rng_eval(1, np.arange(1, 40001), np.full(40000, 7), np.zeros(40000, np.int64)).ravel()
    assert abs(big.mean()) < 0.02 and abs(big.var() - 1.0) < 0.03
    assert abs(np.mean(big ** 4) - 3.0) < 0.1


def _temperature(st, s):
    return 2.0 * st.engke / (BOLTZ * (3 * s.natms - 3 - s.ntcons))


def test_berendsen_pins_temperature_with_tau_equal_to_timestep(oracle_lib):
    s = systems.nacl_melt(16)
    oracle_lib.init(s)
    oracle_lib.start()
    oracle_lib.set_ensemble("berendsen", temp=1000.0, tau_t=s.tstep)
    for st in oracle_lib.md_vv(5):
        assert _temperature(st, s) == pytest.approx(1000.0, rel=1e-12)
    d = oracle_lib.download()
    p = [float(np.sum(s.weight * d[k])) for k in ("vx", "vy", "vz")]
    assert max(abs(x) for x in p) < 1e-8
    assert oracle_lib.thermostat_state()["chi_t"] == pytest.approx(1.0, abs=1e-12)


def test_nose_hoover_conserves_extended_energy(oracle_lib):
    s = systems.nacl_melt(16)
    oracle_lib.init(s)
    oracle_lib.start()
    oracle_lib.set_ensemble("nose-hoover", temp=1200.0, tau_t=0.02)
    st = oracle_lib.md_vv(30)
    h = np.array([x.engcpe_rc + x.engcpe_rl + x.engcpe_ex + x.engvdw + x.engke + x.consv for x in st])
    consv = np.array([x.consv for x in st])
    assert np.ptp(consv) > 100.0 * np.ptp(h)                            # the thermostat does work ...
    assert np.ptp(h) < 1e-4 * abs(h[0])                                 # ... and the extended energy stays
    th = oracle_lib.thermostat_state()
    q = 2.0 * 0.5 * (3 * s.natms - 3) * BOLTZ * 1200.0 * 0.02 ** 2
    assert th["consv"] == pytest.approx(0.5 * q * th["chi_t"] ** 2 + 2.0 * 0.5 * (3 * s.natms - 3) * BOLTZ
                                        * 1200.0 * th["cint"], rel=1e-12)


def test_langevin_is_reproducible_and_cools(oracle_lib):
    s = systems.nacl_melt(16)
    runs = []
    for seed in ((0, 0, 0), (0, 0, 0), (3, 1, 4)):
        oracle_lib.init(s)
        oracle_lib.start()
        oracle_lib.set_ensemble("langevin", temp=300.0, chi=20.0, seed=seed)
        st = oracle_lib.md_vv(15)
        runs.append((oracle_lib.download(), [_temperature(x, s) for x in st]))
    assert np.array_equal(runs[0][0]["x"], runs[1][0]["x"])             # same seed, same trajectory
    assert not np.array_equal(runs[0][0]["x"], runs[2][0]["x"])         # other seed, other noise
    t = runs[0][1]
    assert t[-1] < 0.8 * 1500.0 and t[-1] > 300.0                       # relaxing from 1500 K towards 300 K
    d = runs[0][0]
    assert max(abs(float(np.sum(s.weight * d[k]))) for k in ("vx", "vy", "vz")) < 1e-8


def test_ensemble_arguments_are_checked(oracle_lib):
    s = systems.nacl_melt(16)
    oracle_lib.init(s)
    for kind, kw in (("berendsen", dict(temp=300.0, tau_t=0.0)), ("nose-hoover", dict(temp=0.0, tau_t=0.1)),
                     ("langevin", dict(temp=300.0, chi=-1.0)), (7, dict(temp=300.0))):
        with pytest.raises(Exception):
            oracle_lib.set_ensemble(kind, **kw)
