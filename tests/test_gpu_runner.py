"""Standalone runs from DL_POLY input files on the GPU path, against the same files
run through the oracle: STATIS records, REVCON and REVIVE agree."""
import os

import numpy as np
import pytest

from dlpoly_gb300 import dlpoly_io as io
from dlpoly_gb300 import runner

pytestmark = pytest.mark.gpu


def _statis(path):
    """{step: values} from a STATIS file."""
    rec = open(path).read().split("\n")[2:]
    out, k = {}, 0
    while k < len(rec) and rec[k]:
        step, count = int(rec[k][:10]), int(rec[k][24:34])
        vals = []
        k += 1
        while len(vals) < count:
            vals += [float(x) for x in rec[k].split()]
            k += 1
        out[step] = np.array(vals)
    return out


@pytest.mark.parametrize("workload,steps", [("water_1536", 12), ("nacl_4096", 20)])
def test_runner_gpu_matches_oracle(tmp_path, gpu_lib, oracle_lib, workload, steps):
    dirs = {}
    for name, lib in (("gpu", gpu_lib), ("oracle", oracle_lib)):
        d = str(tmp_path / name)
        runner.emit(workload, d, steps=steps, stats_every=4)
        out = runner.run(d, lib=lib, quiet=True)
        assert out["final_step"] == steps
        dirs[name] = d
    a = _statis(os.path.join(dirs["gpu"], "STATIS"))
    b = _statis(os.path.join(dirs["oracle"], "STATIS"))
    assert sorted(a) == sorted(b) == list(range(0, steps + 1, 4))
    for step in a:
        scale = np.maximum(np.abs(b[step]), 1e-6 * np.abs(b[step]).max())
        # STATIS prints 7 significant digits; the paths agree far below that
        assert np.all(np.abs(a[step] - b[step]) <= 1e-6 * scale + 1e-12), step
    ra = io.read_config(os.path.join(dirs["gpu"], "REVCON"))
    rb = io.read_config(os.path.join(dirs["oracle"], "REVCON"))
    assert ra.step == rb.step == steps
    np.testing.assert_allclose(ra.pos, rb.pos, rtol=0, atol=1e-9 * np.abs(rb.pos).max())
    np.testing.assert_allclose(ra.vel, rb.vel, rtol=0, atol=1e-8 * np.abs(rb.vel).max())
    np.testing.assert_allclose(ra.frc, rb.frc, rtol=0, atol=1e-7 * np.abs(rb.frc).max())
    s = io.system_from_files(ra, io.read_field(os.path.join(dirs["gpu"], "FIELD")),
                             io.read_control(os.path.join(dirs["gpu"], "CONTROL")))
    sa, sb = io.Statistics(s), io.Statistics(s)
    sa.read_revive(os.path.join(dirs["gpu"], "REVIVE"))
    sb.read_revive(os.path.join(dirs["oracle"], "REVIVE"))
    assert sa.numacc == sb.numacc == steps
    np.testing.assert_allclose(sa.sumval, sb.sumval, rtol=1e-6, atol=1e-9 * np.abs(sb.sumval).max())


def test_runner_mixed_form_from_gbcontrol(tmp_path, gpu_lib):
    d = str(tmp_path)
    runner.emit("nacl_4096", d, steps=10, stats_every=5, gb={"gb_precision": "mixed"})
    out = runner.run(d, lib=gpu_lib, quiet=True)
    assert out["precision"] == "mixed" and out["final_step"] == 10
    st = _statis(os.path.join(d, "STATIS"))
    e0, e10 = st[0][0], st[10][0]                       # total energy (kJ/mol)
    assert abs(e10 - e0) < 1e-4 * abs(st[0][2])          # conserved to well below the configurational energy
