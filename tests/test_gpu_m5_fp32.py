"""Model-5 FP32-flux form (FP32 reconstruction, wave speeds and HLLC; FP64 residuals, RK
state and pressure recovery) against the FP64 form.

Bar: relative L1 error of density, mixture pressure and volume fraction against the FP64
form <= 1e-4, or -- where the reference's scheme amplifies rounding-level differences --
no more than 3x the FP64 form's own change when its initial state is perturbed by 1e-7
(relative, seeded).  The reference's model-5 step is discontinuous in rounding-level
quantities (its star-state energy takes (u* + S_K) where HLLC has (S_K - u*), which makes
the left- and right-star energy fluxes differ by ~2 c E A at a face with u* ~ 0, and its
pressure-relaxation Newton iteration stops on a pressure floor for part of the cells), so
on stiff cases the FP64 form itself does not reproduce under 1e-7 perturbations; the
FP32 form is held to that floor there and to 1e-4 where the floor is below it."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, m5_params
from helpers import mesh_from_golden

from forestfv_public_gb300 import FFVError, Solver
from forestfv_public_gb300.fields import error_report

pytestmark = pytest.mark.gpu
BAR = 1e-4
FP32 = 1
PERTURBATION = 1e-7


def run(g, mesh, S_soa, steps, precision, order=None):
    q = m5_params(g)
    s = Solver(model=5, order=order or int(g["order"]), rk_steps=int(g["rk_steps"]),
               gamma=q["gamma"], pinf=q["pinf"], mu=q["mu"], amin=q["amin"],
               avf_lim=q["avf_lim"], prelax=q["prelax"], precision=precision)
    s.set_mesh(mesh)
    s.upload_state(np.ascontiguousarray(S_soa))
    try:
        s.step(float(g["dt"]), steps)
        return s.download_state()
    finally:
        s.close()


def report(g, a, b):
    q = m5_params(g)
    solid = 0 if q["mu"][0] != 0.0 else None
    return error_report(a, b, q["gamma"], q["pinf"], q["mu"], q["amin"], solid=solid)


def errors_and_floor(name, steps, order=None):
    g = load_golden(name)
    m = mesh_from_golden(g)
    S0 = np.ascontiguousarray(g["S_init"].T)
    ref = run(g, m, S0, steps, 0, order)
    rng = np.random.default_rng(11)
    Sp = S0 * (1.0 + PERTURBATION * rng.uniform(-1.0, 1.0, S0.shape))
    floor = report(g, run(g, m, Sp, steps, 0, order), ref)
    S32 = run(g, m, S0, steps, FP32, order)
    assert np.isfinite(S32).all()
    return report(g, S32, ref), floor


def check(err, floor, keys=("rho", "p", "alpha")):
    for key in keys:
        bar = max(BAR, 3.0 * floor[key]["rel_l1"])
        assert err[key]["rel_l1"] <= bar, (key, err, floor)


CASES = [("m5_bubble_prelax3", 1), ("m5_bubble_prelax3", 3), ("m5_mild_prelax1", 3),
         ("m5_mild_prelax1", 6), ("m5_wall_rk3_order1", 3), ("m5_wall_amr", 3),
         ("m5_wall_gfm", 2), ("m5_wall_symmetry", 4)]


@pytest.mark.parametrize("name,steps", CASES)
def test_fp32_form_against_fp64_form(name, steps, built_lib):
    err, floor = errors_and_floor(name, steps)
    check(err, floor)


@pytest.mark.parametrize("name", ["m5_bubble_prelax3", "m5_mild_prelax1"])
def test_fp32_form_first_step_within_bar(name, built_lib):
    """One step from a state at rest, before any rounding-level branch decision: the plain
    1e-4 bar (in practice the error is at FP32 rounding level)."""
    err, _ = errors_and_floor(name, 1)
    for key in ("rho", "p", "alpha"):
        assert err[key]["rel_l1"] <= 1e-6, (key, err)


def test_fp32_form_order1(built_lib):
    err, floor = errors_and_floor("m5_mild_prelax1", 3, order=1)
    check(err, floor)


def test_fp32_form_reports_nan(built_lib):
    """The ghost-fluid fixture's mixture slab blows up a few steps past its end in the
    FP64 form (a NaN wave speed, as in the reference); the FP32 form reports it too."""
    g = load_golden("m5_wall_gfm")
    m = mesh_from_golden(g)
    with pytest.raises(FFVError):
        run(g, m, g["S_init"].T, 3 * int(g["steps"]), FP32)
