import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "dl-poly_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: long-running case")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    return oracle.load()


@pytest.fixture(scope="session")
def gpu_lib():
    import dlpoly_gb300 as gb

    return gb.load()


def forces(d):
    import numpy as np

    return np.stack([d["fx"], d["fy"], d["fz"]], 1)


def force_dev(a, b):
    """max |F_a - F_b| over atoms and components, relative to the rms force of b."""
    import numpy as np

    Fa, Fb = forces(a), forces(b)
    rms = np.sqrt((Fb ** 2).sum(1).mean())
    return float(np.abs(Fa - Fb).max() / rms)


def force_rms_rel(a, b):
    """rms |F_a - F_b| relative to rms |F_b| (the mixed-form error measure)."""
    import numpy as np

    Fa, Fb = forces(a), forces(b)
    return float(np.sqrt(((Fa - Fb) ** 2).sum(1).mean() / (Fb ** 2).sum(1).mean()))
