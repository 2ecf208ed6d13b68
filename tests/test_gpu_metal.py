"""Tabulated EAM metals on the GPU (gb_metal.cu) against the oracle's restatement of
metal_ld_compute / metal_forces, through the C-ABI."""
import numpy as np
import pytest

from conftest import force_dev
from dlpoly_gb300 import systems
from test_metal_oracle import kat_check, poly_tables, two_atoms

pytestmark = pytest.mark.gpu


def test_eam_known_answers_on_gpu(gpu_lib):
    for r in (1.3, 2.7183, 5.9):
        kat_check(gpu_lib, r=r)


@pytest.mark.parametrize("n_side,listed", [(8, None), (10, (1, 0, 1))])
def test_eam_forces_match_oracle(gpu_lib, oracle_lib, n_side, listed):
    s = systems.eam_alloy(n_side)
    if listed is not None:        # the Cu-Ni pair not listed in FIELD 'metal': no cross force
        s.metal_listed = np.array(listed, np.int32)
    for lib in (gpu_lib, oracle_lib):
        lib.init(s)
        lib.start()
    a, b = gpu_lib.download(), oracle_lib.download()
    assert force_dev(a, b) < 1e-10
    ea, eb = gpu_lib.metal_energies(), oracle_lib.metal_energies()
    for k in ("engmet", "engden"):
        assert ea[k] == pytest.approx(eb[k], rel=1e-10), k
    # the virial sums pair repulsion against embedding attraction: cancellation leaves
    # it ~100x smaller than its terms, so its bar is 1e-9
    assert ea["virmet"] == pytest.approx(eb["virmet"], rel=1e-9)
    np.testing.assert_allclose(gpu_lib.metal_rho(), oracle_lib.metal_rho(), rtol=1e-11)


def test_eam_md_matches_oracle(gpu_lib, oracle_lib):
    s = systems.eam_alloy(8)
    for lib in (gpu_lib, oracle_lib):
        lib.init(s)
        lib.start()
    sd, sr = gpu_lib.md_vv(12), oracle_lib.md_vv(12)
    assert [x.list_rebuilt for x in sd] == [x.list_rebuilt for x in sr]
    for x, y in zip(sd, sr):
        assert x.engmet == pytest.approx(y.engmet, rel=1e-10)
        assert x.virmet == pytest.approx(y.virmet, rel=1e-9)
        assert x.engke == pytest.approx(y.engke, rel=1e-10)
    a, b = gpu_lib.download(), oracle_lib.download()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.abs(a[k] - b[k]).max() <= 1e-9 * np.abs(b[k]).max(), k


def test_eam_error_statuses_on_gpu(gpu_lib):
    s = two_atoms(0.9)
    s.eam = poly_tables()
    gpu_lib.init(s)
    with pytest.raises(Exception, match="506"):
        gpu_lib.start()
    s = two_atoms(2.0)
    tabs = poly_tables()
    tabs[2] = dict(tabs[2], start=5.0, finish=10.0)
    s.eam = tabs
    gpu_lib.init(s)
    with pytest.raises(Exception, match="507"):
        gpu_lib.start()
    kat_check(gpu_lib)             # the context is still usable
