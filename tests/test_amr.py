"""Host logic of the adaptive time loop: whether a refineh pass changes any leaf (the early
end of meshadaptation's rounds) and the level the gradient criteria assign."""
import numpy as np

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
