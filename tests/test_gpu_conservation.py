"""Global conservation sums (ffv_conservation_sums) and the conservation they show.

The residual is atomic-free: a 1:1 face's flux is evaluated once by its owner (the earlier
cell) and the later cell takes it negated, so the FP64 sum over cells of |V| S telescopes.
In a box with reflective walls mass and total energy are then conserved to FP64 round-off,
in the FP64 form and in the FP32-flux form alike (the FP32 flux value enters both cells)."""
import numpy as np
import pytest

from conftest import load_golden, m5_params
from helpers import mesh_from_golden

from forestfv_public_gb300 import Mesh, Solver
from forestfv_public_gb300.mesh import uniform_leaves
from forestfv_public_gb300.workloads import mixture_state, random_blast_m0

pytestmark = pytest.mark.gpu
REFLECTIVE = (4,) * 6


def test_sums_reproducible_and_equal_host_sum(built_lib):
    g = load_golden("m5_wall_amr")
    q = m5_params(g)
    s = Solver(model=5, gamma=q["gamma"], pinf=q["pinf"], mu=q["mu"], amin=q["amin"],
               avf_lim=q["avf_lim"], prelax=q["prelax"])
    m = mesh_from_golden(g)
    s.set_mesh(m)
    S = np.ascontiguousarray(g["S_final"].T)
    s.upload_state(S)
    a, b = s.conservation_sums(), s.conservation_sums()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    vol = (0.5 / (1 << (m.level - 1)).astype(np.float64)) ** 3  # 2^3 trees on the unit cube
    ref = (S * vol[None, :]).sum(axis=1)
    scale = (np.abs(S) * vol[None, :]).sum(axis=1) + 1e-300
    assert (np.abs(a - ref) / scale).max() <= 1e-13
    s.close()


def test_model0_mass_energy_conserved_reflective_box(built_lib):
    m = Mesh((4, 4, 4), uniform_leaves((4, 4, 4), 3), bc=REFLECTIVE)
    s = Solver()
    s.set_mesh(m)
    s.upload_state(random_blast_m0(m, 7))
    dt = s.cfl_dt(0.4)
    s0 = s.conservation_sums()
    s.step(dt, 30)
    s1 = s.conservation_sums()
    for v in (0, 4):  # mass, total energy
        assert abs(s1[v] - s0[v]) <= 1e-13 * abs(s0[v]), (v, s0[v], s1[v])
    s.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_model5_partial_masses_conserved_reflective_box(precision, built_lib):
    """A gas bubble in liquid in a closed box: each material's mass is conserved to FP64
    round-off in the FP64 form.  In the FP32-flux form the interior fluxes still cancel
    exactly; what is left is the reflective wall's mass flux rho (S - u)/S S - rho S, zero in
    exact arithmetic and an FP32 rounding of rho S per wall face here (1.6e-12 relative over
    10 steps on this machine)."""
    m = Mesh((2, 2, 2), uniform_leaves((2, 2, 2), 4), bc=REFLECTIVE)
    mat = dict(gamma=(4.4, 1.4), pinf=(6e8, 0.0), rho=(1000.0, 1.0), p=(5e6, 1e5), amin=1e-6)
    x = m.centroids()
    a_gas = 0.5 * (1.0 - np.tanh((np.linalg.norm(x - 0.5, axis=1) - 0.2) / 0.04))
    S = mixture_state(mat, a_gas)
    s = Solver(model=5, gamma=mat["gamma"], pinf=mat["pinf"], mu=(0.0, 0.0), amin=mat["amin"],
               avf_lim=1.0, prelax=3, precision=precision)
    s.set_mesh(m)
    s.upload_state(S)
    dt = 0.01 * (1.0 / 16) / np.sqrt(4.4 * (5e6 + 6e8) / 1000.0)
    s0 = s.conservation_sums()
    s.step(dt, 10)
    s1 = s.conservation_sums()
    tol = 1e-13 if precision == 0 else 1e-10
    for v in (0, 1):  # alpha rho of each material
        assert abs(s1[v] - s0[v]) <= tol * abs(s0[v]), (v, s0[v], s1[v])
    s.close()
