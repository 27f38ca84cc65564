"""Refinement tags, host part: the 2:1 smoothing (ffv_tags_smooth, criterionsmth.c) against
the reference's own smoothing of the same target levels, for every tag pass the model-5
fixtures hold (generated by tests/golden/make_golden.py from the reference's
interface_location / criterionsplt / criterionsmth)."""
import ctypes

import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import mesh_from_golden

from forestfv_public_gb300 import _lib


def level_max(t):
    """LEVEL as inputset.c:106 and m5_input.c:53 form it from the criterion levels."""
    return int(max(t[1], t[3], t[6], t[9], t[12], t[15]))


@pytest.mark.parametrize("name", golden_names(model=5))
def test_smoothing_matches_reference(name, built_lib):
    g = load_golden(name)
    m = mesh_from_golden(g)
    L = _lib.lib()
    assert g["tags"].shape[0] >= 3
    for params, ref in zip(g["tag_params"], g["tags"]):
        split = np.ascontiguousarray(ref[:, 2].astype(np.int32))
        rc = L.ffv_tags_smooth(m.handle, level_max(params), split.ctypes.data)
        assert rc == 0
        assert np.array_equal(split, ref[:, 3]), (name, params)


def test_smoothing_is_two_to_one():
    """After smoothing no face neighbour's target exceeds a leaf's by more than one."""
    from forestfv_public_gb300.mesh import Mesh, uniform_leaves
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 4))
    rng = np.random.default_rng(3)
    split = rng.integers(1, 7, m.n).astype(np.int32)
    assert _lib.lib().ffv_tags_smooth(m.handle, 6, split.ctypes.data) == 0
    ex = m.export()
    nb, bc = ex["nb"], ex["bc"]
    for c in range(m.n):
        for f in range(6):
            if bc[c, f] == 0:
                for q in nb[c, f]:
                    if q >= 0:
                        assert split[q] - split[c] <= 1


def _smooth_sequential(m, lmax, split):
    """criterionsmth.c:3-58 restated plainly: LEVEL + 1 passes of the two in-place sweeps in
    leaf order (coarsen only with all eight sibling leaves, refine by one; at most one level
    below any face neighbour)."""
    split = split.copy()
    n, lev = m.n, m.level
    c_ijk, t_ijk = m.cell_ijk, m.tree_ijk
    kid = ((c_ijk[:, 0] & 1) << 1) | (c_ijk[:, 1] & 1) | ((c_ijk[:, 2] & 1) << 2)
    group = np.full(n, -1)
    for c in range(n):
        s = c - kid[c]
        if lev[c] > 1 and s >= 0 and s + 8 <= n and all(
                lev[s + q] == lev[c] and kid[s + q] == q and (t_ijk[s + q] == t_ijk[c]).all()
                and ((c_ijk[s + q] >> 1) == (c_ijk[c] >> 1)).all() for q in range(8)):
            group[c] = s
    e = m.export()
    nbrs = [[int(e["nb"][c, f, q]) for f in range(6) for q in range(int(e["nn"][c, f]))]
            for c in range(n)]
    for _ in range(lmax + 1):
        for c in range(n):
            l = lev[c]
            if l > 1:
                g = group[c]
                imerge = sum(1 for q in range(g, g + 8) if split[q] < lev[q]) if g >= 0 else 0
                if imerge == 8:
                    split[c] = l - 1
                elif l > split[c]:
                    split[c] = l
            if l < split[c]:
                split[c] = l + 1
        for c in range(n):
            mx = max([1] + [split[d] for d in nbrs[c]])
            if mx - split[c] > 1:
                split[c] = mx - 1
    return split


@pytest.mark.parametrize("seed,mode", [(3, "noise"), (4, "noise"), (5, "noise"),
                                       (6, "groups"), (7, "groups"), (8, "coarsen")])
def test_smoothing_equals_sequential_sweeps(seed, mode, built_lib):
    """The smoothing as built (the coarsening rule's sweep in parallel over sibling groups,
    the 2:1 rule's as a worklist after a parallel evaluation of dirty leaves) against the
    plain sequential sweeps, on random targets of an AMR forest: independent noise per
    leaf, one random offset per group of eight consecutive leaves (whole groups that want
    to coarsen, next to groups that do not), and targets mostly below the level."""
    from forestfv_public_gb300 import Mesh
    from forestfv_public_gb300.solver import tags_smooth
    from forestfv_public_gb300.workloads import refine_to_target
    rng = np.random.default_rng(seed)
    leaves = refine_to_target((2, 2, 2), 2, 4, lambda c, h: np.where(
        c[:, 0] < 0.25, 4, np.where(c[:, 0] < 0.5, 3, 2)))
    m = Mesh((2, 2, 2), leaves)
    lmax = 6
    if mode == "noise":
        d = rng.integers(-2, 3, m.n)
    elif mode == "groups":
        d = np.repeat(rng.integers(-2, 2, (m.n + 7) // 8), 8)[:m.n]
        d = d + (rng.random(m.n) < 0.05) * rng.integers(-1, 2, m.n)
    else:
        d = -rng.integers(0, 3, m.n) + (rng.random(m.n) < 0.02)
    split = np.clip(m.level + d, 1, lmax).astype(np.int32)
    assert np.array_equal(tags_smooth(m, lmax, split), _smooth_sequential(m, lmax, split))
