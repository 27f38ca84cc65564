"""Reference-form geometry of a Cartesian forest, in numpy (TEST INFRASTRUCTURE).

What the reference's own neighbour search and geometry give for a forest of axis-aligned
cubic hex trees -- elconn.c:3-145 (neighbours across levels), meshproperties.c:27-38,
:42-73, :76-124 (centroid, face area as a triangle fan, volume as six tetrahedra),
normalvector.c:15-46 and tagvector.c:60-87 (face frames), distance.c:120-167 (distances) --
in the per-leaf form the CPU restatement takes (oracle/pyoracle.OracleMesh): one row per
cell face, six per cell, cells in the reference's leaf-list order (rebuildlist.c:30-91:
trees in Morton order, then depth-first by child index).

This module loads no compiled code: bench.py's CPU legs use it so that they time the
restatement without mapping the CUDA library, and tests/test_oracle_forest.py checks it
bit for bit against the library's own export of the same forest (ffv_mesh_export).

Hex corner k sits at (x, y, z) = (bit1 k, bit0 k, bit2 k): the node order whose normals
point into the cell and whose six-tet volume is negative, the handedness the reference's
update S = SN - DT/Vol RHS needs to be upwind.
"""
from __future__ import annotations

import numpy as np

# operatetp.c:64-69 (hex faces, typ 0) and operatetp.c:268-279 (opposite face)
FACE_NODES = ((0, 1, 5, 4), (3, 7, 5, 1), (2, 6, 7, 3), (2, 0, 4, 6), (2, 3, 1, 0), (6, 4, 5, 7))
FACE_OPP = (2, 3, 0, 1, 5, 4)
CORNER = np.array([[(k >> 1) & 1, k & 1, (k >> 2) & 1] for k in range(8)], dtype=np.int64)
BC_OUTLET = 2


def _node_pos(h: float) -> list:
    return [tuple(float(CORNER[k][a]) * h for a in range(3)) for k in range(8)]


def _face_frame(nd, f):
    """normalvector.c:23-29 (n = (P1-P0) x (P2-P0) normalised, its components as written
    there) and tagvector.c:69-83 (t1 along the first edge, t2 = n x t1 normalised)."""
    import math
    p0, p1, p2 = nd[FACE_NODES[f][0]], nd[FACE_NODES[f][1]], nd[FACE_NODES[f][2]]
    a = (p1[1] - p0[1]) * (p2[2] - p0[2]) - (p2[1] - p0[1]) * (p1[2] - p0[2])
    b = (p1[0] - p0[0]) * (p2[2] - p0[2]) - (p2[0] - p0[0]) * (p1[2] - p0[2])
    c = (p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1])
    norm = math.sqrt(a * a + b * b + c * c)
    n = (a / norm, -b / norm, c / norm)
    norm = math.sqrt((p1[1] - p0[1]) ** 2 + (p1[0] - p0[0]) ** 2 + (p1[2] - p0[2]) ** 2)
    t1 = ((p1[0] - p0[0]) / norm, (p1[1] - p0[1]) / norm, (p1[2] - p0[2]) / norm)
    a = n[1] * t1[2] - t1[1] * n[2]
    b = n[0] * t1[2] - t1[0] * n[2]
    c = n[0] * t1[1] - t1[0] * n[1]
    norm1 = math.sqrt(a * a + b * b + c * c)
    t2 = (a / norm1, -b / norm1, c / norm1)
    return n + t1 + t2


def _face_area(nd, f):
    """meshproperties.c:61-69: a fan of two triangles from the face's node 0."""
    import math
    area = 0.0
    for it in range(2):
        p0, p1, p2 = nd[FACE_NODES[f][0]], nd[FACE_NODES[f][1 + it]], nd[FACE_NODES[f][2 + it]]
        dx1, dx2 = p1[0] - p0[0], p2[0] - p0[0]
        dy1, dy2 = p1[1] - p0[1], p2[1] - p0[1]
        dz1, dz2 = p1[2] - p0[2], p2[2] - p0[2]
        cx, cy, cz = dy1 * dz2 - dz1 * dy2, dz1 * dx2 - dx1 * dz2, dx1 * dy2 - dy1 * dx2
        area += abs(0.5 * math.sqrt(cx * cx + cy * cy + cz * cz))
    return area


def _hex_volume(nd):
    """meshproperties.c:83-123: the signed volume as six tetrahedra on node 0."""
    vn = ((1, 3, 5), (5, 3, 7), (5, 7, 4), (3, 2, 7), (7, 2, 6), (7, 6, 4))
    vol = 0.0
    for tet in vn:
        dx = [nd[q][0] - nd[0][0] for q in tet]
        dy = [nd[q][1] - nd[0][1] for q in tet]
        dz = [nd[q][2] - nd[0][2] for q in tet]
        c0 = dy[0] * dz[1] - dz[0] * dy[1]
        c1 = dz[0] * dx[1] - dx[0] * dz[1]
        c2 = dx[0] * dy[1] - dy[0] * dx[1]
        vol += (c0 * dx[2] + c1 * dy[2] + c2 * dz[2]) / 6.0
    return vol


def _side(f):
    """(axis, direction) of the domain that face f looks along: the coordinate its four
    nodes share, -1 where they sit at 0, +1 where at 1."""
    bits = CORNER[list(FACE_NODES[f])]
    for a in range(3):
        if (bits[:, a] == bits[0, a]).all():
            return a, (1 if bits[0, a] else -1)
    raise AssertionError("not a hex face")


SIDES = [_side(f) for f in range(6)]
FRAMES = np.array([_face_frame(_node_pos(1.0), f) for f in range(6)])


def _spread3(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
    out = np.zeros_like(v)
    for b in range(21):
        out |= ((v >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b)
    return out


def _morton(x, y, z) -> np.ndarray:
    """Key whose base-8 digits are child indices (x = bit1, y = bit0, z = bit2)."""
    return (_spread3(x) << np.uint64(1)) | _spread3(y) | (_spread3(z) << np.uint64(2))


def leaf_order(tree_ijk, level, cell_ijk) -> np.ndarray:
    """Permutation into the reference's leaf-list order: trees by the Morton key of their
    indices, then depth-first by child index."""
    tree_ijk = np.asarray(tree_ijk, np.int64)
    cell_ijk = np.asarray(cell_ijk, np.int64)
    level = np.asarray(level, np.int64)
    D = int(level.max()) - 1
    sh = (D - (level - 1)).astype(np.uint64)
    tkey = _morton(tree_ijk[:, 0], tree_ijk[:, 1], tree_ijk[:, 2])
    lkey = _morton(cell_ijk[:, 0].astype(np.uint64) << sh, cell_ijk[:, 1].astype(np.uint64) << sh,
                   cell_ijk[:, 2].astype(np.uint64) << sh)
    return np.lexsort((level, lkey, tkey))


class Forest:
    """The leaves of a Cartesian forest in leaf-list order, with a lookup of leaves by
    (level, global cell coordinates)."""

    def __init__(self, ntrees, tree_ijk, level, cell_ijk, bc=(BC_OUTLET,) * 6,
                 tree_edge: float | None = None, ordered: bool = False):
        self.ntrees = np.asarray(ntrees, np.int64)
        self.bc = tuple(int(b) for b in bc)
        self.tree_edge = float(tree_edge if tree_edge is not None else 1.0 / self.ntrees.max())
        perm = np.arange(len(level)) if ordered else leaf_order(tree_ijk, level, cell_ijk)
        self.order = perm
        self.tree_ijk = np.asarray(tree_ijk, np.int64)[perm]
        self.cell_ijk = np.asarray(cell_ijk, np.int64)[perm]
        self.level = np.asarray(level, np.int64)[perm]
        self.n = len(self.level)
        self.gx = self.tree_ijk * (1 << (self.level - 1))[:, None] + self.cell_ijk
        key = self._key(self.level, self.gx)
        self._ks = np.argsort(key)
        self._key_sorted = key[self._ks]
        self.geom = {}
        for lv in range(1, int(self.level.max()) + 2):
            h = self.tree_edge / float(1 << (lv - 1))
            nd = _node_pos(h)
            self.geom[lv] = (h, _hex_volume(nd), _face_area(nd, 0))

    @staticmethod
    def _key(level, g):
        g = np.asarray(g)
        return (np.asarray(level, np.uint64) << np.uint64(60)) | _morton(g[..., 0], g[..., 1], g[..., 2])

    def find(self, level, g) -> np.ndarray:
        """Cell index of the leaf at (level, global coordinates g), -1 where there is none."""
        key = self._key(level, g)
        pos = np.searchsorted(self._key_sorted, key)
        pos = np.minimum(pos, len(self._key_sorted) - 1)
        hit = self._key_sorted[pos] == key
        return np.where(hit, self._ks[pos], -1)

    def centroids(self, cells=None) -> np.ndarray:
        c = np.arange(self.n) if cells is None else np.asarray(cells)
        h = self.tree_edge / (1 << (self.level[c] - 1)).astype(np.float64)
        return self.tree_ijk[c] * self.tree_edge + (self.cell_ijk[c] + 0.5) * h[:, None]

    def geometry(self, cells=None) -> dict:
        """Reference-form geometry of `cells` (all when None; an increasing index array
        keeps the leaf-list order) as one mesh of its own: neighbours are renumbered into
        the selection, and a face whose neighbour (or any of whose four finer neighbours)
        lies outside the selection becomes a transmissive boundary face.  Keys and shapes
        as the library's Mesh.export()."""
        cells = np.arange(self.n) if cells is None else np.asarray(cells, np.int64)
        m = len(cells)
        local = np.full(self.n, -1, np.int64)
        local[cells] = np.arange(m)
        lev = self.level[cells]
        gx = self.gx[cells]
        out = dict(bc=np.zeros((m, 6), np.int32), nn=np.zeros((m, 6), np.int32),
                   neigfc=np.tile(np.array(FACE_OPP, np.int32), (m, 1)),
                   nb=np.full((m, 6, 4), -1, np.int32), area=np.zeros((m, 6, 4)),
                   nrm=np.tile(FRAMES[None], (m, 1, 1)), dist_cf=np.zeros((m, 6)),
                   dist_cc=np.zeros((m, 6)))
        hl = np.array([self.geom[lv][0] for lv in range(1, int(lev.max()) + 2)])
        vol_l = np.array([self.geom[lv][1] for lv in range(1, int(lev.max()) + 2)])
        area_l = np.array([self.geom[lv][2] for lv in range(1, int(lev.max()) + 2)])
        h = hl[lev - 1]
        out["vol"] = vol_l[lev - 1]
        lo = self.tree_ijk[cells] * self.tree_edge + self.cell_ijk[cells] * h[:, None]
        out["centroid"] = (4.0 * lo + 4.0 * (lo + h[:, None])) / 8.0
        for f in range(6):
            a, d = SIDES[f]
            g = gx.copy()
            g[:, a] += d
            ext = self.ntrees[a] << (lev - 1)
            outside = (g[:, a] < 0) | (g[:, a] >= ext)
            same = np.where(outside, -1, self.find(lev, np.clip(g, 0, None)))
            coarse = np.where(outside | (same >= 0) | (lev <= 1), -1,
                              self.find(lev - 1, np.clip(g, 0, None) >> 1))
            fine = np.full((m, 4), -1, np.int64)
            need = ~outside & (same < 0) & (coarse < 0)
            if need.any():
                for k in range(4):
                    q = FACE_NODES[f][k]
                    fg = 2 * g[need]
                    for b in range(3):
                        fg[:, b] += (0 if d > 0 else 1) if b == a else CORNER[q][b]
                    fine[need, k] = self.find(lev[need] + 1, fg)
                if (fine[need] < 0).any():
                    raise ValueError("forest has a hole or violates 2:1 balance")
            # renumber into the selection; a neighbour outside it makes a boundary face
            same_l = np.where(same >= 0, local[np.maximum(same, 0)], -1)
            coarse_l = np.where(coarse >= 0, local[np.maximum(coarse, 0)], -1)
            fine_l = np.where(fine >= 0, local[np.maximum(fine, 0)], -1)
            is_same = same_l >= 0
            is_coarse = coarse_l >= 0
            is_fine = need & (fine_l >= 0).all(axis=1)
            is_bc = ~(is_same | is_coarse | is_fine)
            side = 2 * a + (1 if d > 0 else 0)
            out["bc"][:, f] = np.where(outside, self.bc[side], np.where(is_bc, BC_OUTLET, 0))
            out["nn"][:, f] = np.where(is_fine, 4, np.where(is_same | is_coarse, 1, 0))
            out["nb"][:, f, 0] = np.where(is_same, same_l, np.where(is_coarse, coarse_l, -1))
            out["nb"][is_fine, f, :] = fine_l[is_fine]
            out["area"][:, f, 0] = np.where(is_fine, area_l[np.minimum(lev, len(area_l) - 1)],
                                            area_l[lev - 1])
            for k in range(1, 4):
                out["area"][:, f, k] = np.where(is_fine, area_l[np.minimum(lev, len(area_l) - 1)],
                                                0.0)
            # distance.c:120-167 by neighbour relation (0 on boundary faces)
            hp = hl[np.maximum(lev - 2, 0)]
            out["dist_cf"][:, f] = np.where(is_same, 0.5 * h, np.where(
                is_fine, 0.5 * h, np.where(is_coarse, 0.25 * hp, 0.0)))
            out["dist_cc"][:, f] = np.where(is_same, h, np.where(
                is_fine, 0.5 * h + 0.25 * h, np.where(is_coarse, 0.25 * hp + 0.5 * hp, 0.0)))
        return out
