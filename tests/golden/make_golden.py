"""Generate the committed golden fixtures from the CPU FP64 oracle.

The reference (Fortran) cannot run here, so the fixtures are the oracle's
output on seeded inputs; they pin the oracle against regressions and give the
GPU tests committed vectors to compare with.  The reference's own known answer
(source/unit_tests/test_vdw.F90:46-59) is checked separately in
tests/test_oracle.py.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "dl-poly_gb300"))

import oracle  # noqa: E402
from dlpoly_gb300 import systems  # noqa: E402

CASES = {
    "nacl_4096": lambda: systems.nacl_melt(16),
    "water_1536": lambda: systems.spce_water(8),
}


def run_case(name, make, nsteps=5):
    o = oracle.load()
    s = make()
    o.init(s)
    o.relocate()
    lst = o.link_cell_pairs()
    e0, st0 = o.two_body_forces()
    d0 = o.download()
    stats = o.md_vv(nsteps)
    d1 = o.download()
    out = dict(
        list_count=lst[:, 3].astype(np.int32),
        list_excl_end=lst[:, 2].astype(np.int32),
        list_checksum=np.array([int(np.sum(lst[:, 4:].astype(np.int64) * (1 + np.arange(lst.shape[1] - 4))))]),
        f0=np.stack([d0["fx"], d0["fy"], d0["fz"]], 1),
        eng0=np.array([e0[k] for k in sorted(e0)]),
        eng_keys=np.array(sorted(e0)),
        stress0=st0,
        x5=np.stack([d1["x"], d1["y"], d1["z"]], 1),
        v5=np.stack([d1["vx"], d1["vy"], d1["vz"]], 1),
        engke=np.array([s_.engke for s_ in stats]),
        shake_iters=np.array([s_.shake_iters for s_ in stats]),
        rattle_iters=np.array([s_.rattle_iters for s_ in stats]),
        rebuilt=np.array([s_.list_rebuilt for s_ in stats]),
    )
    o.finalize()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "written")


if __name__ == "__main__":
    for name, make in CASES.items():
        run_case(name, make)
