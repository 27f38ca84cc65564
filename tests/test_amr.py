"""Host logic of the adaptive time loop: whether a refineh pass changes any leaf (the early
end of meshadaptation's rounds) and the level the gradient criteria assign."""
import numpy as np
import pytest

from forestfv_public_gb300 import Mesh
from forestfv_public_gb300._lib import TagParams
from forestfv_public_gb300.amr import gradient_level
from forestfv_public_gb300.mesh import uniform_leaves
from forestfv_public_gb300.solver import level_max, would_change


def test_would_change_refine_and_merge(built_lib):
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 3))
    lev = m.level.copy()
    assert not would_change(m, lev)
    s = lev.copy()
    s[17] += 1
    assert would_change(m, s)
    # seven of eight siblings coarser: no merge
    s = lev.copy()
    s[8:15] -= 1
    assert not would_change(m, s)
    s[15] -= 1
    assert would_change(m, s)
    # eight consecutive leaves that are not one sibling group do not merge
    s = lev.copy()
    s[4:12] -= 1
    assert not would_change(m, s)


def test_would_change_level_one_trees_never_merge(built_lib):
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 1))
    assert not would_change(m, np.zeros(m.n, np.int32))


def test_gradient_level():
    p = TagParams.from_tuple((1, 3, 1, 5, 0.1, 1, 6, 0.1, 0, 0, 0.0, 1, 7, 2, 0, 0, 0))
    assert gradient_level(p) == 6
    assert level_max(p) == 7
    p = TagParams.from_tuple((1, 3, 0, 0, 0.0, 0, 0, 0.0, 0, 0, 0.0, 1, 7, 2, 0, 0, 0))
    assert gradient_level(p) == 7


def test_carry_marks_children_and_parents():
    from forestfv_public_gb300.amr import carry_marks
    marks = np.array([0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 1], bool)
    # old leaf 0 split into 8, old 1..8 merged into one parent, 9 and 10 kept
    src = np.array([0] * 8 + [-1 - 1] + [9, 10], np.int64)
    got = carry_marks(src, marks)
    assert got.tolist() == [False] * 8 + [True, False, True]
    src = np.array([-1 - 2, 10], np.int64)  # old 2..9 merged (none marked), 10 kept
    assert carry_marks(src, marks).tolist() == [False, True]


def _random_pass(m, rng, lmax):
    from forestfv_public_gb300.solver import tags_smooth
    tgt = m.level + rng.integers(-1, 2, m.n)
    tgt = np.clip(tgt, 1, lmax).astype(np.int32)
    return tags_smooth(m, lmax, tgt)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mesh_adapt_equals_full_build(seed, built_lib):
    """The incremental rebuild of a refineh pass gives the full builder's tables."""
    from forestfv_public_gb300.mesh import Leaves
    from forestfv_public_gb300.solver import mesh_adapt
    from forestfv_public_gb300.workloads import refine_to_target
    rng = np.random.default_rng(seed)
    leaves = refine_to_target((2, 3, 2), 2, 4, lambda c, h: np.where(
        c[:, 0] < 0.25, 4, np.where(c[:, 0] < 0.5, 3, 2)))
    m = Mesh((2, 3, 2), leaves, bc=(2, 4, 1, 2, 3, 2), tree_edge=0.5)
    for _ in range(4):
        split = _random_pass(m, rng, 6)
        new, src = mesh_adapt(m, split)
        ref = Mesh(m.ntrees, Leaves(new.tree_ijk, new.level, new.cell_ijk), bc=m.bc,
                   tree_edge=m.tree_edge)
        assert np.array_equal(ref.order, np.arange(new.n))  # emitted in leaf order
        e1, e2 = new.export(), ref.export()
        for k in e1:
            assert np.array_equal(e1[k], e2[k]), k
        # sources: kept and split leaves point at their old leaf, merged parents at 8 siblings
        lev_old = m.level
        keep = src >= 0
        assert np.all((new.level[keep] == lev_old[src[keep]]) | (new.level[keep] == lev_old[src[keep]] + 1))
        assert np.all(new.level[~keep] == lev_old[-1 - src[~keep]] - 1)
        m = new


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_round_end_check_from_old_levels(seed, built_lib):
    """The learned regrid ends its rounds when no new leaf from an old one is below the old
    leaf's target.  It decides that from the old levels alone (a leaf splits exactly when its
    target is above its level, one level at a time): any(target > level + 1).  Both forms
    agree on smoothed random passes and on passes that split isolated leaves of a uniform
    mesh with targets one or two levels up."""
    from forestfv_public_gb300.mesh import uniform_leaves
    from forestfv_public_gb300.solver import mesh_adapt, tags_smooth
    from forestfv_public_gb300.workloads import refine_to_target
    rng = np.random.default_rng(seed)

    def agree(m, tgt):
        new, src = mesh_adapt(m, tgt)
        keep = src >= 0
        by_src = bool(np.any(tgt[src[keep]] > new.level[keep]))
        assert by_src == bool(np.any(tgt > m.level + 1))
        return new, by_src

    leaves = refine_to_target((2, 2, 2), 2, 4, lambda c, h: np.where(c[:, 0] < 0.5, 4, 3))
    m = Mesh((2, 2, 2), leaves)
    for _ in range(4):
        tgt = tags_smooth(m, 7, np.clip(m.level + rng.integers(-2, 4, m.n), 1, 7).astype(np.int32))
        m, _ = agree(m, tgt)
    u = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 3))
    for up in (1, 2):
        tgt = u.level.astype(np.int32).copy()
        pick = rng.choice(u.n, 6, replace=False)
        tgt[pick] += rng.integers(1, up + 1, 6)
        tgt[pick[0]] = u.level[pick[0]] + up
        _, deeper = agree(u, tgt)
        assert deeper == (up == 2)
