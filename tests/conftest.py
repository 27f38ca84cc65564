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


def golden_names(with_geometry=None, model=None):
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        name = os.path.splitext(os.path.basename(p))[0]
        z = np.load(p)
        if with_geometry is not None and ("nb" in z.files) != with_geometry:
            continue
        if model is not None and int(z["model"]) != model:
            continue
        out.append(name)
    return out


def m5_params(g):
    """Model-5 material parameters of a fixture, as oracle/pyoracle.m5_advance takes them."""
    return dict(avf_lim=float(g["m5_avf_lim"]), prelax=int(g["m5_prelax"]),
                amin=float(g["m5_amin"]), pinf=list(g["m5_pinf"]), gamma=list(g["m5_gamma"]),
                mu=list(g["m5_mu"]))


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
