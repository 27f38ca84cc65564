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


def test_carry_marks_children_and_parents(built_lib):
    from forestfv_public_gb300.amr import carry_marks, morton_intervals
    from forestfv_public_gb300.workloads import refine_to_target
    m0 = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 3))
    a, b = morton_intervals(m0)
    assert np.all(a[1:] == b[:-1])  # leaf order tiles the Morton line
    x0 = m0.centroids()
    marks = (x0[:, 0] < 0.25) & (x0[:, 1] < 0.25) & (x0[:, 2] < 0.25)
    leaves = refine_to_target((2, 2, 2), 2, 4, lambda c, h: np.where(c[:, 0] < 0.25, 4,
                                                                     np.where(c[:, 0] < 0.5, 3, 2)))
    m1 = Mesh((2, 2, 2), leaves)
    a1, b1 = morton_intervals(m1)
    assert np.all(a1[1:] == b1[:-1])
    got = carry_marks(m0, marks, m1)
    x1 = m1.centroids()
    h1 = 0.5 / (1 << (m1.level - 1))
    # a new leaf overlaps the marked box [0, 0.25)^3 exactly when its lower corner is inside
    exp = np.all(x1 - 0.5 * h1[:, None] < 0.25 - 1e-12, axis=1)
    assert np.array_equal(got, exp)
