"""A sheared solid block for the plasticity tests: the wall configuration's solid below
z = 0.5 and liquid above, at rest at 5 MPa on the 8^3 forest, the solid's deformation tensor
carrying a shear A[0][1] = 0.02 sin(2 pi x) (von Mises stress up to 0.83 GPa, above the
configuration's 0.3 GPa yield stress)."""
import numpy as np

from forestfv_public_gb300 import workloads as W
from forestfv_public_gb300.mesh import uniform_leaves
from oracle.forest import Forest

YIELD = 3e8


def sheared_block():
    lv = uniform_leaves((2, 2, 2), 3)
    F = Forest((2, 2, 2), lv.tree_ijk, lv.level, lv.cell_ijk)
    x = F.centroids()
    solid = x[:, 2] < 0.5
    S = W.wall_state(W.WALL, solid, np.zeros(F.n))
    S[12 + 1] = np.where(solid, 0.02 * np.sin(2 * np.pi * x[:, 0]), 0.0)
    m5 = dict(avf_lim=W.WALL["avf_lim"], prelax=3, amin=W.WALL["amin"], pinf=list(W.WALL["pinf"]),
              gamma=list(W.WALL["gamma"]), mu=list(W.WALL["mu"]))
    dt = 0.03 * 0.125 / np.sqrt(3.5 * (5e6 + 3.2e10) / 2700.0)
    return lv, F, S, solid, m5, dt


def von_mises(S, m5):
    from forestfv_public_gb300.fields import primitives
    return primitives(S, m5["gamma"], m5["pinf"], m5["mu"], m5["amin"])["vm"]
