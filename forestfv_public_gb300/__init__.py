"""GB300-native explicit finite-volume step of ForestFV on a forest of octrees.

The compute path is hand-written sm_103a CUDA behind the C ABI of include/ffv.h; this
package is a thin host-side mirror of that ABI (no CPU fallback).
"""
from ._lib import FFV_FLUX_CONSISTENT, FFV_FLUX_REFERENCE, FFV_FP32_FLUX, FFV_FP64, FFVError  # noqa: F401
from .mesh import (BC_INLET, BC_OUTLET, BC_REFLECTIVE, BC_SYMMETRY, BC_WALL, Leaves, Mesh,  # noqa: F401
                   leaves_from_paths, morton_tree_order, uniform_leaves)
from .solver import Solver  # noqa: F401
