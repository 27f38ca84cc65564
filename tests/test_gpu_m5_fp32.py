"""Model-5 FP32-flux form (FP32 reconstruction, wave speeds and HLLC; FP64 residuals, RK
state and pressure recovery) against the FP64 form on the fixtures' meshes.

Quantities: relative L1 error of density, mixture pressure and volume fraction, and the
relative error of the peak wall stress (largest von Mises stress where the solid fraction
exceeds 0.5) on the cases with a solid.

With the consistent flux form (FFV_FLUX_CONSISTENT) the density and the peak wall stress are
held to the metric's bar, 1e-4; the wall stress error is taken relative to the larger of the
peak and 1e-6 of the solid's shear modulus (a strain of 1e-6, ~16 FP32 ulps of the
deformation tensor): the fixtures at rest have peaks of 1e-3 Pa, which are rounding noise.  With the reference's own m5 flux the FP64 form itself does
not reproduce under a 1e-7 perturbation of its initial state on the stiff cases (its star-state
energy takes (u* + S_K) where HLLC has (S_K - u*): a face at rest carries a spurious energy
flux of ~2 c E A whose sign follows rounding noise), so there every quantity, the wall
stress included, is held to 3x that floor where the floor exceeds 1e-4, and to 1e-4 where it
does not; the first step from rest is held to 1e-6."""
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


def run(g, mesh, S_soa, steps, precision, order=None, flux_form=0):
    q = m5_params(g)
    s = Solver(model=5, order=order or int(g["order"]), rk_steps=int(g["rk_steps"]),
               gamma=q["gamma"], pinf=q["pinf"], mu=q["mu"], amin=q["amin"],
               avf_lim=q["avf_lim"], prelax=q["prelax"], precision=precision,
               flux_form=flux_form)
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


def errors_and_floor(name, steps, order=None, flux_form=0):
    g = load_golden(name)
    m = mesh_from_golden(g)
    S0 = np.ascontiguousarray(g["S_init"].T)
    ref = run(g, m, S0, steps, 0, order, flux_form)
    rng = np.random.default_rng(11)
    Sp = S0 * (1.0 + PERTURBATION * rng.uniform(-1.0, 1.0, S0.shape))
    floor = report(g, run(g, m, Sp, steps, 0, order, flux_form), ref)
    S32 = run(g, m, S0, steps, FP32, order, flux_form)
    assert np.isfinite(S32).all()
    return report(g, S32, ref), floor


def check(err, floor, keys=("rho", "p", "alpha")):
    for key in keys:
        bar = max(BAR, 3.0 * floor[key]["rel_l1"])
        assert err[key]["rel_l1"] <= bar, (key, err, floor)
    if "peak_wall_stress" in err:
        bar = max(BAR, 3.0 * floor["peak_wall_stress"]["rel_err"])
        assert err["peak_wall_stress"]["rel_err"] <= bar, (err, floor)


CASES = [("m5_bubble_prelax3", 1), ("m5_bubble_prelax3", 3), ("m5_mild_prelax1", 3),
         ("m5_mild_prelax1", 6), ("m5_wall_rk3_order1", 3), ("m5_wall_amr", 3),
         ("m5_wall_gfm", 2), ("m5_wall_symmetry", 4)]


@pytest.mark.parametrize("name,steps", CASES)
def test_fp32_form_against_fp64_form(name, steps, built_lib):
    err, floor = errors_and_floor(name, steps)
    check(err, floor)


def wall_err(g, err):
    """|peak32 - peak64| / max(peak64, 1e-6 mu_solid)."""
    w = err["peak_wall_stress"]
    scale = max(abs(w["ref"]), 1e-6 * max(m5_params(g)["mu"]))
    return abs(w["test"] - w["ref"]) / scale


@pytest.mark.parametrize("name,steps", CASES)
def test_fp32_form_consistent_flux_within_bar(name, steps, built_lib):
    """The consistent flux form: density and peak wall stress within the metric's bar."""
    err, _ = errors_and_floor(name, steps, flux_form=1)
    assert err["rho"]["rel_l1"] <= BAR, err
    if "peak_wall_stress" in err:
        assert wall_err(load_golden(name), err) <= BAR, err


@pytest.mark.parametrize("name,steps", [("m5_wall_amr", 3), ("m5_wall_rk3_order1", 3)])
def test_fp32_form_consistent_wall_stress_tight(name, steps, built_lib):
    """The deformation carried as A - I: on the wall fixtures the FP32 form's peak wall stress
    stays within 1e-6 of the FP64 form's (measured 1.6e-9 and 2.0e-8; with an FP32 A the
    stress carried ~mu 1e-7 of rounding)."""
    err, _ = errors_and_floor(name, steps, flux_form=1)
    assert wall_err(load_golden(name), err) <= 1e-6, err


@pytest.mark.parametrize("name", ["m5_wall_amr", "m5_wall_rk3_order1"])
def test_fp32_form_wall_first_step_within_bar(name, built_lib):
    """One step from rest on the wall cases, consistent flux: density and the peak wall
    stress within 1e-4."""
    err, _ = errors_and_floor(name, 1, flux_form=1)
    assert err["rho"]["rel_l1"] <= BAR, err
    assert wall_err(load_golden(name), err) <= BAR, err


def test_fp32_form_wall_first_step_reference_flux(built_lib):
    """One step from rest with the reference's flux: within 1e-4 on the first-order case."""
    err, _ = errors_and_floor("m5_wall_rk3_order1", 1)
    assert err["rho"]["rel_l1"] <= BAR, err
    assert wall_err(load_golden("m5_wall_rk3_order1"), err) <= BAR, err


@pytest.mark.xfail(strict=True, reason="the reference's star-state energy is -rho E at rest, "
                   "and its FP32 rounding on the 5e10 J/m^3 solid energy moves the second-order "
                   "case's peak wall stress by 0.92 relative in one step (density 2.1e-6)")
def test_fp32_form_wall_first_step_reference_flux_amr(built_lib):
    err, _ = errors_and_floor("m5_wall_amr", 1)
    assert err["rho"]["rel_l1"] <= BAR and wall_err(load_golden("m5_wall_amr"), err) <= BAR, err


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
