"""Model-5 CUDA path (multi-material flow, hyperelastic solid, ghost-fluid coupling,
pressure relaxation) against the reference's output and the CPU restatement.

Tolerance: 1e-12 relative L-inf per conserved variable (the plain FP64 form's bar).  The
kernels keep the reference's operation order; pow() is the one function whose CUDA and
glibc results can differ in the last bit, so equality is not required here."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, m5_params
from helpers import mesh_from_golden, rel_linf

from forestfv_public_gb300 import Solver
from oracle import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12


def solver_for(g):
    q = m5_params(g)
    return Solver(model=5, order=int(g["order"]), rk_steps=int(g["rk_steps"]), gamma=q["gamma"],
                  pinf=q["pinf"], mu=q["mu"], amin=q["amin"], avf_lim=q["avf_lim"],
                  prelax=q["prelax"])


def run_gpu(g, mesh, S_aos, steps):
    s = solver_for(g)
    s.set_mesh(mesh)
    s.upload_state(np.ascontiguousarray(S_aos.T))
    s.step(float(g["dt"]), steps)
    out = s.download_state().T.copy()
    s.close()
    return out


def scaled_err(out, ref):
    """Per-variable error relative to the variable's magnitude; variables that are zero in
    the reference everywhere (e.g. the deformation tensor in fluid-only cases) are
    compared against the largest state magnitude of their group instead."""
    return rel_linf(out, ref)


@pytest.mark.parametrize("name", golden_names(model=5))
def test_m5_gpu_matches_reference_fixture(name, built_lib):
    g = load_golden(name)
    m = mesh_from_golden(g)
    out = run_gpu(g, m, g["S_init"], int(g["steps"]))
    err = scaled_err(out, g["S_final"])
    assert (err <= TOL).all(), (err.max(), int(err.argmax()))


@pytest.mark.parametrize("name,mult", [("m5_wall_amr", 3), ("m5_bubble_prelax3", 4),
                                       ("m5_mild_prelax1", 4), ("m5_wall_symmetry", 3)])
def test_m5_gpu_matches_oracle_longer(name, mult, built_lib, oracle_lib):
    """More steps than the fixture holds, against the CPU restatement (the ghost-fluid
    fixture's mixture slab stops being a valid state soon after its 4 steps: the
    reference exits there with a NaN wave speed, as the restatement does)."""
    g = load_golden(name)
    m = mesh_from_golden(g)
    steps = mult * int(g["steps"])
    ref = pyoracle.m5_advance(pyoracle.OracleMesh(m.export()), g["S_init"], float(g["dt"]),
                              steps, m5_params(g), int(g["order"]), int(g["rk_steps"]))
    out = run_gpu(g, m, g["S_init"], steps)
    err = rel_linf(out, ref)
    assert (err <= TOL).all(), (err.max(), int(err.argmax()))


def test_m5_nan_wave_speed_reported(built_lib):
    """Where the reference exits (m5_wave_speeds.c:78-129) the device status reports it."""
    from forestfv_public_gb300 import FFVError
    g = load_golden("m5_wall_gfm")
    m = mesh_from_golden(g)
    s = solver_for(g)
    s.set_mesh(m)
    s.upload_state(np.ascontiguousarray(g["S_init"].T))
    with pytest.raises(FFVError) as e:
        s.step(float(g["dt"]), 3 * int(g["steps"]))
    assert e.value.code == 5


@pytest.mark.parametrize("precision", [0, 1])
def test_m5_negative_density_reported(precision, built_lib):
    """A negative partial density injected on the host (both forms): FFV_ERR_NEG_DENSITY."""
    from forestfv_public_gb300 import FFVError
    g = load_golden("m5_wall_amr")
    m = mesh_from_golden(g)
    q = m5_params(g)
    s = Solver(model=5, order=int(g["order"]), rk_steps=int(g["rk_steps"]), gamma=q["gamma"],
               pinf=q["pinf"], mu=q["mu"], amin=q["amin"], avf_lim=q["avf_lim"],
               prelax=q["prelax"], precision=precision)
    s.set_mesh(m)
    S = np.ascontiguousarray(g["S_init"].T).copy()
    S[:3, 40] = -S[:3, 40]
    s.upload_state(S)
    with pytest.raises(FFVError) as e:
        s.step(float(g["dt"]), 1)
    assert e.value.code == 6
    s.close()


def test_cfl_dt_model5(built_lib):
    """ffv_cfl_dt (warp-shuffle min-reduction) against the host restatement:
    dt = cfl * min over cells of h / (max_a |u_a| + c), c^2 = sum_k alpha_k gamma_k
    (p_k + p_inf_k) / rho (the mixture sound speed of m5_wave_speeds.c:43-50)."""
    from forestfv_public_gb300.fields import primitives
    g = load_golden("m5_bubble_prelax3")
    q = m5_params(g)
    m = mesh_from_golden(g)
    s = Solver(model=5, gamma=q["gamma"], pinf=q["pinf"], mu=q["mu"], amin=q["amin"],
               avf_lim=q["avf_lim"], prelax=q["prelax"])
    s.set_mesh(m)
    S = np.ascontiguousarray(g["S_final"].T)
    s.upload_state(S)
    N = len(q["gamma"])
    pr = primitives(S, q["gamma"], q["pinf"], q["mu"], q["amin"])
    gam, pinf = np.asarray(q["gamma"]), np.asarray(q["pinf"])
    p_k = np.stack([(gam[k] - 1.0) * S[2 * N + 3 + k] / pr["alpha"][k] - gam[k] * pinf[k]
                    for k in range(N)])
    c2 = (pr["alpha"] * gam[:, None] * (p_k + pinf[:, None])).sum(axis=0) / pr["rho"]
    u = np.abs(S[N:N + 3] / pr["rho"]).max(axis=0)
    h = 0.5 / (1 << (m.level - 1)).astype(np.float64)
    ref = 0.3 * (h / (u + np.sqrt(c2))).min()
    assert abs(s.cfl_dt(0.3) - ref) <= 1e-10 * ref
    s.close()
