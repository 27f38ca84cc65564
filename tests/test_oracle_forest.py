"""The oracle's numpy forest geometry (oracle/forest.py) against the reference's own geometry
dumps and against the library's export of the same forest, bit for bit; and the geometry of
a contiguous range of leaves as a mesh of its own (the CPU baseline's sample)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from helpers import geometry_from_golden, mesh_from_golden

from forestfv_public_gb300 import leaves_from_paths
from oracle.forest import Forest

KEYS = ("bc", "nn", "neigfc", "nb", "area", "nrm", "dist_cf", "dist_cc", "vol")


def forest_of(g):
    lv = leaves_from_paths(tuple(g["ntrees"]), g["root"], g["level"],
                           g["adrs"][:, 2:].astype(np.int64))
    return Forest(tuple(g["ntrees"]), lv.tree_ijk, lv.level, lv.cell_ijk,
                  bc=tuple(int(b) for b in g["bc_sides"]))


@pytest.mark.parametrize("name", golden_names(with_geometry=True))
def test_forest_geometry_equals_reference_dump(name):
    """The reference's own neighbour search and geometry (dumped by the reference binary
    when the fixture was made): identical in leaf order, neighbours and every double."""
    g = load_golden(name)
    F = forest_of(g)
    assert np.array_equal(F.order, np.arange(F.n))
    geo, ref = F.geometry(), geometry_from_golden(g)
    interior = geo["nn"] > 0
    for k in KEYS:
        if k in ("dist_cf", "dist_cc") and int(g["order"]) == 1:
            continue  # first order: the reference never computes distances (grad_scheme.c)
        a, b = np.asarray(geo[k]).reshape(np.shape(ref[k])), ref[k]
        if k == "neigfc":  # not read on boundary faces, where the reference leaves it unset
            a, b = a[interior], b[interior]
        assert np.array_equal(a, b), k


def test_forest_geometry_equals_library_export(built_lib):
    import bench
    for wl in ("config3", "config2"):
        mesh = bench.WORKLOADS[wl](small=True)[0]
        F = Forest(mesh.ntrees, mesh.tree_ijk, mesh.level, mesh.cell_ijk, bc=mesh.bc)
        ex, geo = mesh.export(), F.geometry()
        for k in KEYS + ("centroid",):
            assert np.array_equal(ex[k], geo[k]), (wl, k)


def test_workload_leaves_without_the_library(built_lib):
    """The CPU legs build the wall configuration's leaves and state in numpy alone: same
    leaf order and initial state as the library-built mesh."""
    from forestfv_public_gb300 import workloads as W
    mesh, S, _ = W.bubble_wall_config3(lmax=5, band_cells=2.0)
    leaves, state = W.bubble_wall_parts(lmax=5, band_cells=2.0)
    F = Forest((2, 2, 2), leaves.tree_ijk, leaves.level, leaves.cell_ijk)
    assert np.array_equal(F.order, mesh.order)
    assert np.array_equal(state(F.centroids()), S)


def test_range_geometry_is_a_mesh_of_its_own():
    """A contiguous range of leaves: neighbours inside renumbered, faces to leaves outside
    transmissive boundaries, everything else as in the whole forest's geometry."""
    g = load_golden("m5_wall_amr")
    F = forest_of(g)
    full = F.geometry()
    a, b = F.n // 3, 2 * F.n // 3
    sel = np.arange(a, b)
    part = F.geometry(sel)
    nb_full = full["nb"][sel]
    inside = (nb_full >= a) & (nb_full < b)
    kept = (full["nn"][sel] > 0) & (inside | (nb_full < 0)).all(axis=2)
    assert np.array_equal(part["nb"][kept], np.where(nb_full[kept] >= 0, nb_full[kept] - a, -1))
    cut = (full["nn"][sel] > 0) & ~kept
    assert cut.any()
    assert (part["bc"][cut] == 2).all() and (part["nn"][cut] == 0).all()
    assert (part["nb"][cut] == -1).all() and (part["dist_cf"][cut] == 0).all()
    assert np.array_equal(part["vol"], full["vol"][sel])
    assert np.array_equal(part["nrm"], full["nrm"][sel])
