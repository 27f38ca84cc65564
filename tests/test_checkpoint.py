"""Checkpoint/restart and field export on the host (no GPU).

* The binary checkpoint round-trips leaves and state bit for bit, rejects a corrupted or
  truncated file, and rebuilds the same face tables.
* The text restart writer is byte-identical to the reference's own restart_save output
  (golden file written by the reference for the fixture's final state), and the reader
  recovers the reference's leaf list and its state to the file's eleven digits.
* The Tecplot writer shares nodes between leaves and writes one brick per leaf."""
import os

import numpy as np
import pytest

from conftest import load_golden
from helpers import mesh_from_golden

from forestfv_public_gb300 import Mesh
from forestfv_public_gb300._lib import FFVError
from forestfv_public_gb300.checkpoint import (load_checkpoint, read_restart_text, save_checkpoint,
                                              write_restart_text, write_tecplot)
from forestfv_public_gb300.mesh import uniform_leaves
from forestfv_public_gb300.workloads import refine_to_target

RESTART_CASES = ("m0_sphere_amr", "m5_wall_amr")


def amr_mesh():
    leaves = refine_to_target((2, 2, 2), 2, 4,
                              lambda c, h: np.where(c[:, 0] < 0.25, 4, np.where(c[:, 0] < 0.5, 3, 2)))
    return Mesh((2, 2, 2), leaves, bc=(2, 4, 2, 1, 3, 2))


def test_checkpoint_roundtrip_bit_exact(tmp_path, built_lib):
    m = amr_mesh()
    rng = np.random.default_rng(3)
    S = rng.standard_normal((21, m.n)) * 10.0 ** rng.integers(-12, 12, (21, m.n))
    p = str(tmp_path / "a.ffvc")
    save_checkpoint(p, m, S, istep=1234, time=5.5e-7)
    m2, S2, istep, t = load_checkpoint(p)
    assert (istep, t) == (1234, 5.5e-7)
    assert m2.ntrees == m.ntrees and m2.bc == m.bc and m2.tree_edge == m.tree_edge
    assert np.array_equal(m2.level, m.level)
    assert np.array_equal(m2.tree_ijk, m.tree_ijk) and np.array_equal(m2.cell_ijk, m.cell_ijk)
    assert np.array_equal(S2.view(np.uint64), S.view(np.uint64))
    e1, e2 = m.export(), m2.export()
    for k in e1:
        assert np.array_equal(e1[k], e2[k]), k


def test_checkpoint_rejects_corruption(tmp_path, built_lib):
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 2))
    p = str(tmp_path / "b.ffvc")
    save_checkpoint(p, m, np.ones((5, m.n)))
    raw = bytearray(open(p, "rb").read())
    raw[200] ^= 0x40
    bad = str(tmp_path / "bad.ffvc")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(FFVError):
        load_checkpoint(bad)
    short = str(tmp_path / "short.ffvc")
    open(short, "wb").write(bytes(raw[:150]))
    with pytest.raises(FFVError):
        load_checkpoint(short)


@pytest.mark.parametrize("name", RESTART_CASES)
def test_restart_text_matches_reference(name, tmp_path, built_lib):
    g = load_golden(name)
    ref_text = bytes(g["restart_text"]).decode("ascii")
    m = mesh_from_golden(g)
    S = np.ascontiguousarray(g["S_final"].T)
    istep = int(g["steps"])
    t = float(g["dt"]) * istep
    p = str(tmp_path / "restart.dat")
    write_restart_text(p, m, S, istep=istep, time=t)
    assert open(p).read() == ref_text
    # read the reference's file back: its leaves, the state to eleven digits
    rp = str(tmp_path / "ref.dat")
    open(rp, "w").write(ref_text)
    m2, S2, istep2, t2 = read_restart_text(rp, tuple(g["ntrees"]), tuple(g["bc_sides"]))
    assert istep2 == istep and abs(t2 - t) <= 1e-10 * abs(t)
    assert np.array_equal(m2.level, m.level)
    assert np.array_equal(m2.tree_ijk, m.tree_ijk) and np.array_equal(m2.cell_ijk, m.cell_ijk)
    assert np.allclose(S2, S, rtol=1e-10, atol=1e-300)


def test_restart_text_roundtrip_amr(tmp_path, built_lib):
    m = amr_mesh()
    rng = np.random.default_rng(4)
    S = rng.uniform(-2, 2, (5, m.n))
    p = str(tmp_path / "r.dat")
    write_restart_text(p, m, S, 7, 0.25)
    m2, S2, istep, t = read_restart_text(p, m.ntrees, m.bc)
    assert (istep, t) == (7, 0.25)
    assert np.array_equal(m2.level, m.level) and np.array_equal(m2.cell_ijk, m.cell_ijk)
    assert np.allclose(S2, S, rtol=1e-10)


def test_tecplot_shares_nodes(tmp_path, built_lib):
    m = amr_mesh()
    x = m.centroids()
    p = str(tmp_path / "f.plt")
    write_tecplot(p, m, {"x": x[:, 0], "lvl": m.level.astype(float)}, time=1.0)
    lines = open(p).read().split("\n")
    assert lines[1].startswith('VARIABLES = "X" "Y" "Z" "x" "lvl"')
    z = lines[2]
    assert "ZONETYPE=FEBRICK" in z and "VARLOCATION=([4-5]=CELLCENTERED)" in z
    nn = int(z.split("N=")[1].split(",")[0])
    ne = int(z.split("E=")[1].split(",")[0])
    assert ne == m.n
    # every distinct lattice point of the leaves' corners is one node
    L = int(m.level.max())
    corners = set()
    for c in range(m.n):
        l = int(m.level[c])
        s = 1 << (L - l)
        g = (m.tree_ijk[c].astype(np.int64) << (l - 1)) + m.cell_ijk[c]
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    corners.add(tuple(((g + (dx, dy, dz)) * s).tolist()))
    assert nn == len(corners)
    conn = [list(map(int, ln.split())) for ln in lines if ln.strip() and len(ln.split()) == 8
            and all(t.isdigit() for t in ln.split())]
    assert len(conn) == m.n and max(max(r) for r in conn) == nn and min(min(r) for r in conn) == 1
