"""Shared helpers for the tests: fixture -> mesh / geometry / state conversions."""
import numpy as np

from forestfv_public_gb300 import Mesh, leaves_from_paths


def mesh_from_golden(g):
    leaves = leaves_from_paths(tuple(g["ntrees"]), g["root"], g["level"],
                               g["adrs"][:, 2:].astype(np.int64))
    m = Mesh(tuple(g["ntrees"]), leaves, bc=tuple(int(b) for b in g["bc_sides"]))
    assert np.array_equal(m.order, np.arange(m.n)), "leaf order differs from the reference's"
    return m


def geometry_from_golden(g):
    return dict(bc=g["bc"], nn=g["nn"], neigfc=g["neigfc"], nb=g["nb"], area=g["area"],
                nrm=g["nrm"].astype(np.float64), dist_cf=g["dist_cf"], dist_cc=g["dist_cc"],
                vol=g["vol"])


def rel_linf(a, b):
    """Per-variable max |a-b| / max |b| (AoS [n, neq])."""
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return np.abs(a - b).max(axis=0) / scale
