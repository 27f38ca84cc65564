import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def golden_names(with_geometry=None):
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        name = os.path.splitext(os.path.basename(p))[0]
        if with_geometry is not None:
            has = "nb" in np.load(p).files
            if has != with_geometry:
                continue
        out.append(name)
    return out


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="session")
def built_lib():
    """The in-tree CUDA library (mesh builder + kernels); built if missing."""
    from forestfv_public_gb300 import build
    if not os.path.exists(build.LIB):
        build.build()
    return build.LIB


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import pyoracle
    pyoracle.build()
    return pyoracle
