"""Forest description and face tables (host side), over ffv_mesh_build / ffv_mesh_export.

A forest is ntrees[0] x ntrees[1] x ntrees[2] cubic hex trees; a leaf is (tree index,
level, integer coordinates inside the tree).  Trees are level 1 and a leaf at level l has
2**(l-1) cells per tree edge, as in the reference (spawntopo.c:136, split.c:25).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib

BC_SYMMETRY, BC_OUTLET, BC_INLET, BC_REFLECTIVE, BC_WALL = 1, 2, 3, 4, 5

# corner k of a hex sits at (x, y, z) = (bit1(k), bit0(k), bit2(k)) (see ffv_internal.h)
CORNER = np.array([[(k >> 1) & 1, k & 1, (k >> 2) & 1] for k in range(8)], dtype=np.int32)


@dataclass
class Leaves:
    tree_ijk: np.ndarray  # [n,3] int32
    level: np.ndarray     # [n]   int32
    cell_ijk: np.ndarray  # [n,3] int32

    @property
    def n(self) -> int:
        return int(self.level.shape[0])


def uniform_leaves(ntrees: tuple[int, int, int], level: int) -> Leaves:
    """Every tree refined uniformly to `level`."""
    e = 1 << (level - 1)
    t = np.stack(np.meshgrid(*[np.arange(k, dtype=np.int32) for k in ntrees], indexing="ij"),
                 -1).reshape(-1, 3)
    c = np.stack(np.meshgrid(*[np.arange(e, dtype=np.int32)] * 3, indexing="ij"), -1).reshape(-1, 3)
    tree = np.repeat(t, len(c), axis=0)
    cell = np.tile(c, (len(t), 1))
    lev = np.full(len(tree), level, dtype=np.int32)
    return Leaves(tree.astype(np.int32), lev, cell.astype(np.int32))


def leaves_from_paths(ntrees, tree_index, level, paths) -> Leaves:
    """Leaves given as the reference addresses them: tree index in Morton order of the
    tree coordinates and the child indices from level 2 down (BRANCH.adrs, split.c:31-34)."""
    order = morton_tree_order(ntrees)
    n = len(level)
    tree = order[np.asarray(tree_index)]
    cell = np.zeros((n, 3), dtype=np.int32)
    lev = np.asarray(level, dtype=np.int32)
    for i in range(n):
        for k in paths[i][: lev[i] - 1]:
            cell[i] = cell[i] * 2 + CORNER[k]
    return Leaves(tree.astype(np.int32), lev, cell)


def _spread3(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
    out = np.zeros_like(v)
    for b in range(21):
        out |= ((v >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b)
    return out


def morton_tree_order(ntrees) -> np.ndarray:
    """Tree coordinates sorted in the leaf-list order (child-index Morton order)."""
    t = np.stack(np.meshgrid(*[np.arange(k) for k in ntrees], indexing="ij"), -1).reshape(-1, 3)
    key = (_spread3(t[:, 0]) << np.uint64(1)) | _spread3(t[:, 1]) | (_spread3(t[:, 2]) << np.uint64(2))
    return t[np.argsort(key, kind="stable")].astype(np.int32)


class Mesh:
    """Owner-sorted face tables built by the library (ffv_mesh_build)."""

    def __init__(self, ntrees, leaves: Leaves, bc=(BC_OUTLET,) * 6, tree_edge: float | None = None,
                 part: bool = False):
        """part: the leaves are a part of a forest (ffv_mesh_build_part): faces towards
        leaves that are not among them become transmissive boundaries."""
        L = _lib.lib()
        self.ntrees = tuple(int(t) for t in ntrees)
        self.bc = tuple(int(b) for b in bc)
        self.tree_edge = float(tree_edge if tree_edge is not None else 1.0 / max(self.ntrees))
        d = _lib.ForestDesc()
        d.ntrees[:] = self.ntrees
        d.bc[:] = self.bc
        d.tree_edge = self.tree_edge
        tij = np.ascontiguousarray(leaves.tree_ijk, dtype=np.int32)
        lev = np.ascontiguousarray(leaves.level, dtype=np.int32)
        cij = np.ascontiguousarray(leaves.cell_ijk, dtype=np.int32)
        self._order = np.zeros(leaves.n, dtype=np.int64)
        h = ctypes.c_void_p()
        build = L.ffv_mesh_build_part if part else L.ffv_mesh_build
        _lib.check(build(ctypes.byref(d), leaves.n, tij.ctypes.data, lev.ctypes.data,
                         cij.ctypes.data, ctypes.byref(h), self._order.ctypes.data),
                   "ffv_mesh_build")
        self._h = h
        self.n = int(L.ffv_mesh_ncells(h))
        self.level = lev[self._order]
        self._coords = (tij[self._order], cij[self._order])

    @classmethod
    def from_handle(cls, h, ntrees, bc, tree_edge) -> "Mesh":
        """Wrap tables the library built itself (ffv_adapt)."""
        L = _lib.lib()
        m = cls.__new__(cls)
        m.ntrees, m.bc, m.tree_edge = tuple(ntrees), tuple(bc), float(tree_edge)
        m._h = h
        m.n = int(L.ffv_mesh_ncells(h))
        m.level = np.empty(m.n, np.int32)
        _lib.check(L.ffv_mesh_leaves(h, None, m.level.ctypes.data, None), "ffv_mesh_leaves")
        m._coords = None  # the leaves' coordinates, copied on first use
        m._order = None
        return m

    def _leaf_coords(self):
        if self._coords is None:
            t = np.empty((self.n, 3), np.int32)
            c = np.empty((self.n, 3), np.int32)
            _lib.check(_lib.lib().ffv_mesh_leaves(self._h, t.ctypes.data, None, c.ctypes.data),
                       "ffv_mesh_leaves")
            self._coords = (t, c)
        return self._coords

    @property
    def tree_ijk(self) -> np.ndarray:
        return self._leaf_coords()[0]

    @property
    def cell_ijk(self) -> np.ndarray:
        return self._leaf_coords()[1]

    @property
    def order(self) -> np.ndarray:
        """Leaf-list position of each input leaf (the identity for tables the library
        built itself)."""
        if self._order is None:
            self._order = np.arange(self.n, dtype=np.int64)
        return self._order

    @property
    def handle(self):
        return self._h

    def export(self) -> dict:
        """Reference-form geometry (see ffv_mesh_export)."""
        n = self.n
        out = dict(bc=np.zeros((n, 6), np.int32), nn=np.zeros((n, 6), np.int32),
                   neigfc=np.zeros((n, 6), np.int32), nb=np.zeros((n, 6, 4), np.int32),
                   area=np.zeros((n, 6, 4)), nrm=np.zeros((n, 6, 9)), dist_cf=np.zeros((n, 6)),
                   dist_cc=np.zeros((n, 6)), vol=np.zeros(n), centroid=np.zeros((n, 3)))
        keys = ("bc", "nn", "neigfc", "nb", "area", "nrm", "dist_cf", "dist_cc", "vol", "centroid")
        _lib.check(_lib.lib().ffv_mesh_export(self._h, *[out[k].ctypes.data for k in keys]),
                   "ffv_mesh_export")
        return out

    def centroids(self) -> np.ndarray:
        h = self.tree_edge / (1 << (self.level - 1)).astype(np.float64)
        return self.tree_ijk * self.tree_edge + (self.cell_ijk + 0.5) * h[:, None]

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().ffv_mesh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
