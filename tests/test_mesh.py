"""Host face-table builder: ordering, validation and error codes (no GPU)."""
import numpy as np
import pytest

from forestfv_public_gb300 import FFVError, Leaves, Mesh, uniform_leaves


def test_uniform_counts_and_order(built_lib):
    lv = uniform_leaves((2, 2, 2), 3)
    rng = np.random.default_rng(0)
    perm = rng.permutation(lv.n)
    shuffled = Leaves(lv.tree_ijk[perm], lv.level[perm], lv.cell_ijk[perm])
    m = Mesh((2, 2, 2), shuffled)
    assert m.n == 8 * 64
    e = m.export()
    assert (e["nn"][e["bc"] == 0] == 1).all()
    assert (e["bc"] != 0).sum() == 6 * 8 * 8
    # canonical order does not depend on input order
    m2 = Mesh((2, 2, 2), lv)
    assert np.array_equal(m.tree_ijk, m2.tree_ijk) and np.array_equal(m.cell_ijk, m2.cell_ijk)


def test_overlap_rejected(built_lib):
    lv = uniform_leaves((1, 1, 1), 2)
    bad = Leaves(np.vstack([lv.tree_ijk, [[0, 0, 0]]]).astype(np.int32),
                 np.append(lv.level, 1).astype(np.int32),
                 np.vstack([lv.cell_ijk, [[0, 0, 0]]]).astype(np.int32))
    with pytest.raises(FFVError) as e:
        Mesh((1, 1, 1), bad)
    assert e.value.code == 3


def test_unbalanced_rejected(built_lib):
    # one tree at level 1 next to a tree refined to level 3: 2:1 violated
    a = uniform_leaves((1, 1, 1), 3)
    tree = np.vstack([np.zeros((a.n, 3), np.int32), [[1, 0, 0]]]).astype(np.int32)
    lev = np.append(a.level, 1).astype(np.int32)
    cell = np.vstack([a.cell_ijk, [[0, 0, 0]]]).astype(np.int32)
    with pytest.raises(FFVError) as e:
        Mesh((2, 1, 1), Leaves(tree, lev, cell))
    assert e.value.code == 4


def test_hole_rejected(built_lib):
    a = uniform_leaves((1, 1, 1), 2)
    keep = np.arange(a.n) != 3
    with pytest.raises(FFVError) as e:
        Mesh((1, 1, 1), Leaves(a.tree_ijk[keep], a.level[keep], a.cell_ijk[keep]))
    assert e.value.code in (3, 4)


def test_out_of_range_rejected(built_lib):
    with pytest.raises(FFVError):
        Mesh((1, 1, 1), Leaves(np.array([[0, 0, 0]], np.int32), np.array([2], np.int32),
                               np.array([[2, 0, 0]], np.int32)))


def test_mesh_leaves_partial_outputs(built_lib):
    """ffv_mesh_leaves fills any subset of its three outputs (a library-built mesh copies its
    leaf coordinates only when asked) and refuses a call that asks for none."""
    import numpy as np

    from forestfv_public_gb300 import _lib
    from forestfv_public_gb300.mesh import Mesh, uniform_leaves
    m = Mesh((2, 1, 1), uniform_leaves((2, 1, 1), 3))
    L = _lib.lib()
    lev = np.zeros(m.n, np.int32)
    assert L.ffv_mesh_leaves(m.handle, None, lev.ctypes.data, None) == 0
    assert np.array_equal(lev, m.level)
    t = np.zeros((m.n, 3), np.int32)
    c = np.zeros((m.n, 3), np.int32)
    assert L.ffv_mesh_leaves(m.handle, t.ctypes.data, None, c.ctypes.data) == 0
    assert np.array_equal(t, m.tree_ijk) and np.array_equal(c, m.cell_ijk)
    assert L.ffv_mesh_leaves(m.handle, None, None, None) == 1  # FFV_ERR_ARG
    wrapped = Mesh.from_handle(m.handle, m.ntrees, m.bc, m.tree_edge)
    assert np.array_equal(wrapped.level, m.level)
    assert np.array_equal(wrapped.tree_ijk, m.tree_ijk)
    assert np.array_equal(wrapped.cell_ijk, m.cell_ijk)
    wrapped._h = None  # the handle stays owned by m
