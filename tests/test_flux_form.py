"""Model 5's consistent flux form (FFV_FLUX_CONSISTENT) in the CPU restatement.

The reference's m5 flux is kept to the last bit by default; three of its expressions
disagree with the rest of its HLLC solver (the star-state energy of m5_star_region.c:59,
the momentum-flux sign of m5_flux.c:20-34, the left/right deformation-flux sign of
m5_flux.c:53-56).  These tests show what that does and what the consistent form restores:
model 5 with two identical ideal gases solves Sod's problem as model 0 does, a
solid-liquid interface at rest stays at rest, and a 1e-7 perturbation of the wall
configuration's state is not amplified."""
import numpy as np
import pytest

from forestfv_public_gb300 import workloads as W
from forestfv_public_gb300.mesh import uniform_leaves
from oracle import pyoracle
from oracle.forest import Forest

GAS2 = dict(avf_lim=1.0, prelax=3, amin=1e-6, pinf=[0.0, 0.0], gamma=[1.4, 1.4], mu=[0.0, 0.0])


def uniform_forest(level):
    lv = uniform_leaves((2, 2, 2), level)
    return Forest((2, 2, 2), lv.tree_ijk, lv.level, lv.cell_ijk)


def sod_states(F):
    """Sod's problem along x as model-0 [5, n] and model-5 [18, n] (two ideal gases with
    gamma 1.4, the first at volume fraction 1 - 1e-6) states."""
    x = F.centroids()
    left = x[:, 0] < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    S0 = np.zeros((5, F.n))
    S0[0], S0[4] = rho, p / 0.4
    a0, a1 = 1.0 - 1e-6, 1e-6
    S5 = np.zeros((18, F.n))
    S5[0], S5[1] = a0 * rho, a1 * rho
    S5[5] = p / 0.4
    S5[6] = a0
    S5[7], S5[8] = a0 * p / 0.4, a1 * p / 0.4
    return S0, S5


def test_reference_form_fails_sods_problem(oracle_lib):
    """As written, the reference's model 5 stops on Sod's problem after one step (NaN wave
    speed: m5_flux.c pushes the gas with the negated pressure)."""
    F = uniform_forest(4)
    om = pyoracle.OracleMesh(F.geometry())
    _, S5 = sod_states(F)
    dt = 0.4 * (1.0 / 16.0) / np.sqrt(1.4)
    with pytest.raises(RuntimeError, match="code 2"):
        pyoracle.m5_advance(om, S5.T, dt, 3, dict(GAS2, flux_form=0))


def test_consistent_form_solves_sods_problem_as_model0(oracle_lib):
    F = uniform_forest(4)
    om = pyoracle.OracleMesh(F.geometry())
    S0, S5 = sod_states(F)
    dt = 0.4 * (1.0 / 16.0) / np.sqrt(1.4)
    m0 = pyoracle.m0_advance(om, S0.T, dt, 20).T
    m5 = pyoracle.m5_advance(om, S5.T, dt, 20, dict(GAS2, flux_form=1)).T
    for a, b in ((m5[0] + m5[1], m0[0]), (m5[2], m0[1]), (m5[5], m0[4])):
        assert np.abs(a - b).sum() / np.abs(b).sum() < 1e-4
    assert np.abs(m0[1]).max() > 0.2  # the waves have moved


def rest_interface():
    """Solid below z = 0.5, liquid above, both at rest at 5 MPa (the wall configuration's
    materials) on the 8^3 forest."""
    F = uniform_forest(3)
    x = F.centroids()
    S = W.wall_state(W.WALL, x[:, 2] < 0.5, np.zeros(F.n))
    m5 = dict(avf_lim=W.WALL["avf_lim"], prelax=3, amin=W.WALL["amin"], pinf=list(W.WALL["pinf"]),
              gamma=list(W.WALL["gamma"]), mu=list(W.WALL["mu"]))
    dt = 0.03 * 0.125 / np.sqrt(3.5 * (5e6 + 3.2e10) / 2700.0)
    return pyoracle.OracleMesh(F.geometry()), S, m5, dt


def test_consistent_form_keeps_an_interface_at_rest(oracle_lib):
    om, S, m5, dt = rest_interface()
    out = pyoracle.m5_advance(om, S.T, dt, 3, dict(m5, flux_form=1)).T
    assert np.abs(out[6] - S[6]).max() / np.abs(S[6]).max() < 1e-10  # total energy
    assert np.abs(out[3:6]).max() < 1e-3  # momentum, kg / (m^2 s)


def test_reference_form_moves_an_interface_at_rest(oracle_lib):
    """The reference's star-state energy is -rho E at u* = 0: the boundary faces of a state
    at rest change its energy by percents per step."""
    om, S, m5, dt = rest_interface()
    out = pyoracle.m5_advance(om, S.T, dt, 3, dict(m5, flux_form=0)).T
    assert np.abs(out[6] - S[6]).max() / np.abs(S[6]).max() > 1e-2


def test_consistent_form_does_not_amplify_rounding(oracle_lib, built_lib):
    """The wall configuration's sample (levels 4-5): a 1e-7 relative perturbation of the
    initial state stays at that size after 20 steps (the reference's form turns it into
    ~1e-3 in density within 10 steps)."""
    import bench
    from forestfv_public_gb300.fields import error_report
    mesh, S0, dt, _, kw, _, _ = bench.wl_config3(small=True)
    om = pyoracle.OracleMesh(mesh.export())
    m5 = dict(avf_lim=kw["avf_lim"], prelax=kw["prelax"], amin=kw["amin"], pinf=list(kw["pinf"]),
              gamma=list(kw["gamma"]), mu=list(kw["mu"]), flux_form=1)
    rng = np.random.default_rng(3)
    Sp = S0 * (1.0 + 1e-7 * rng.uniform(-1.0, 1.0, S0.shape))
    a = pyoracle.m5_advance(om, S0.T, dt, 20, m5).T
    b = pyoracle.m5_advance(om, Sp.T, dt, 20, m5).T
    e = error_report(b, a, kw["gamma"], kw["pinf"], kw["mu"], kw["amin"], 0)
    assert e["rho"]["rel_l1"] < 2e-7, e
