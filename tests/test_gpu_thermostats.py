"""NVT thermostats on the GPU (gb_thermostat.cu) against the oracle's stages
(nvt_b0_vv, nvt_h0_vv, nvt_l0_vv), through the C-ABI, and the device random
stream against the oracle's sarurnd / box_mueller_saru3."""
import numpy as np
import pytest

from conftest import force_dev
from dlpoly_gb300 import systems

pytestmark = pytest.mark.gpu

CASES = {"nacl_4096": (lambda: systems.nacl_melt(16), 16), "water_1536": (lambda: systems.spce_water(8), 12)}
ENS = {
    "berendsen": dict(temp=900.0, tau_t=0.05),
    "nose-hoover": dict(temp=900.0, tau_t=0.05),
    "langevin": dict(temp=900.0, chi=5.0, seed=(2, 7, 1)),
}


def test_device_random_stream_matches_oracle(gpu_lib, oracle_lib):
    gpu_lib.init(systems.nacl_melt(16))
    rng = np.random.default_rng(3)
    a = rng.integers(1, 1 << 31, 20000)
    b = rng.integers(-(1 << 31), 1 << 31, 20000)
    c = rng.integers(0, 16, 20000)
    assert np.array_equal(gpu_lib.rng_eval(0, a, b, c), oracle_lib.rng_eval(0, a, b, c))   # bit-exact
    c[:] = 0
    gd, go = gpu_lib.rng_eval(1, a, b, c), oracle_lib.rng_eval(1, a, b, c)
    # the uniforms are bit-exact; log/sqrt of the device library may differ by an ulp
    assert np.max(np.abs(gd - go) / np.maximum(np.abs(go), 1e-300)) < 1e-14


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("ens", list(ENS))
def test_thermostat_stages_match_oracle(gpu_lib, oracle_lib, case, ens):
    make, nsteps = CASES[case]
    s = make()
    for lib in (gpu_lib, oracle_lib):
        lib.init(s)
        lib.start()
        lib.set_ensemble(ens, **ENS[ens])
    sd = gpu_lib.md_vv(nsteps)
    sr = oracle_lib.md_vv(nsteps)
    assert [x.list_rebuilt for x in sd] == [x.list_rebuilt for x in sr]
    assert [x.shake_iters for x in sd] == [x.shake_iters for x in sr]
    for x, y in zip(sd, sr):
        assert x.engke == pytest.approx(y.engke, rel=1e-9)
        assert x.consv == pytest.approx(y.consv, rel=1e-9, abs=1e-9 * abs(y.engke))
    a, b = gpu_lib.download(), oracle_lib.download()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.abs(a[k] - b[k]).max() <= 1e-9 * np.abs(b[k]).max(), k
    assert force_dev(a, b) < 1e-8
    ta, tb = gpu_lib.thermostat_state(), oracle_lib.thermostat_state()
    for k in ("chi_t", "cint"):
        assert ta[k] == pytest.approx(tb[k], rel=1e-9, abs=1e-12)


def test_langevin_gpu_reproducible_and_step_keyed(gpu_lib):
    """The mixed form sums forces in fixed point, so a Langevin run repeats bit for
    bit; starting at another step number draws other noise."""
    s = systems.nacl_melt(16)
    out = []
    for start in (0, 0, 100):
        gpu_lib.init(s, precision=1)
        gpu_lib.start()
        gpu_lib.set_ensemble("langevin", temp=600.0, chi=10.0)
        gpu_lib.set_step(start)
        gpu_lib.md_vv(5)
        out.append(gpu_lib.download()["vx"])
    assert np.array_equal(out[0], out[1])
    assert np.abs(out[0] - out[2]).max() > 0.1 * np.abs(out[0]).max()   # the noise is keyed on the step
