"""The bench's own configurations on the GPU against the oracle, and the metric's accuracy
condition for the FP32-flux form.

Parity: the plain FP64 form on the small sizes of the wall (config 3: three materials, a
hyperelastic solid, ghost-fluid faces, levels 4-5) and bubble (config 2: two materials,
levels 4-6) meshes, with the reference's m5 flux and with the consistent flux form, against
the CPU restatement in the same form: 1e-12 relative L-inf per conserved variable.

Accuracy condition (the metric's): relative L1 error of density and relative error of the
peak wall stress (the largest von Mises stress over cells whose solid fraction exceeds 0.5)
of the FP32-flux form against the FP64 form, each <= 1e-4, on the medium wall mesh (0.41 M
cells, levels 4-7), where the wall stress after 20 steps at CFL 0.1 is a physical 4.6 MPa.  With the
consistent flux form it holds; with the reference's own flux it does not (the reference's
star-state energy amplifies rounding differences by ~1e9 within 20 steps), which the
expected failure below records with its measured numbers."""
import numpy as np
import pytest

import bench
from forestfv_public_gb300 import Solver
from forestfv_public_gb300.fields import error_report
from oracle import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12
BAR = 1e-4


def dt_for(workload, dt, flux_form):
    """The wall configurations run at CFL 0.1; with the reference's own flux at 0.01, where its
    scheme stays finite."""
    if workload.startswith("config3") and flux_form == 0:
        return dt * bench.REFERENCE_FLUX_CFL / bench.WALL_CFL
    return dt


def solver(kw, precision, flux_form, mesh, S0):
    s = Solver(precision=precision, flux_form=flux_form, **kw)
    s.set_mesh(mesh)
    s.upload_state(S0)
    return s


@pytest.mark.parametrize("flux_form", [0, 1])
@pytest.mark.parametrize("workload", ["config3", "config2"])
def test_fp64_small_config_matches_oracle(workload, flux_form, built_lib, oracle_lib):
    mesh, S0, dt, _, kw, _, _ = bench.WORKLOADS[workload](small=True)
    dt = dt_for(workload, dt, flux_form)
    s = solver(kw, 0, flux_form, mesh, S0)
    s.step(dt, 3)
    out = s.download_state()
    s.close()
    m5 = dict(avf_lim=kw["avf_lim"], prelax=kw["prelax"], amin=kw["amin"], pinf=list(kw["pinf"]),
              gamma=list(kw["gamma"]), mu=list(kw["mu"]), flux_form=flux_form,
              **{"yield": list(kw.get("yield_stress") or ())})
    ref = pyoracle.m5_advance(pyoracle.OracleMesh(mesh.export()), S0.T, dt, 3, m5).T
    scale = np.maximum(np.abs(ref).max(axis=1), 1e-300)
    err = np.abs(out - ref).max(axis=1) / scale
    assert (err <= TOL).all(), (err.max(), int(err.argmax()))
    assert np.abs(out - S0).max() > 0  # the state moved


def fp32_against_fp64(flux_form, steps, cfl=bench.WALL_CFL):
    mesh, S0, dt, _, kw, _, _ = bench.wl_config3(medium=True)
    dt = dt * cfl / bench.WALL_CFL
    a, b = solver(kw, 0, flux_form, mesh, S0), solver(kw, 1, flux_form, mesh, S0)
    a.step(dt, steps)
    b.step(dt, steps)
    e = error_report(b.download_state(), a.download_state(), kw["gamma"], kw["pinf"], kw["mu"],
                     kw["amin"], solid=0)
    a.close()
    b.close()
    return e


@pytest.mark.parametrize("steps", [20, 100])
def test_fp32_form_meets_the_accuracy_condition(steps, built_lib):
    e = fp32_against_fp64(1, steps)
    assert e["peak_wall_stress"]["ref"] > 1e5  # a physical wall stress, not noise
    assert e["rho"]["rel_l1"] <= BAR, e
    assert e["peak_wall_stress"]["rel_err"] <= BAR, e


@pytest.mark.xfail(strict=True, reason="the reference's m5 flux amplifies rounding-level "
                   "differences: measured on this mesh, density 1.7e-3 and peak wall stress "
                   "6.3e-3 after 20 steps (3.7e-5 and 6.0e-2 after 5)")
def test_fp32_form_with_the_reference_flux_misses_the_accuracy_condition(built_lib):
    e = fp32_against_fp64(0, 20, cfl=bench.REFERENCE_FLUX_CFL)
    assert e["rho"]["rel_l1"] <= BAR and e["peak_wall_stress"]["rel_err"] <= BAR, e


@pytest.mark.parametrize("flux_form", [0, 1])
@pytest.mark.parametrize("workload", ["config3", "config2"])
def test_tags_on_small_config_match_restatement(workload, flux_form, built_lib):
    """The bench's criteria (uniform level 4, relative density jump 0.1 and 16 interface
    layers to the finest level) on the state after 3 FP64 steps: the GPU's interface layers,
    raw and smoothed target levels equal the reference's tag passes as restated in
    oracle/tags.py (pinned against the reference in tests/test_oracle_tags.py)."""
    from oracle import tags as T
    mesh, S0, dt, _, kw, _, _ = bench.WORKLOADS[workload](small=True)
    dt = dt_for(workload, dt, flux_form)
    s = solver(kw, 0, flux_form, mesh, S0)
    s.step(dt, 3)
    S = s.download_state()
    t = bench.wall_tags(int(mesh.level.max()))
    split, raw, si = s.tags(t, with_raw=True)
    s.close()
    m5 = dict(avf_lim=kw["avf_lim"], amin=kw["amin"], pinf=list(kw["pinf"]),
              gamma=list(kw["gamma"]), mu=list(kw["mu"]))
    SI, raw_r, split_r = T.tags(S, mesh.export(), m5, t, mesh.level, mesh.tree_ijk,
                                mesh.cell_ijk)
    assert np.array_equal(si[0], SI[0]) and np.array_equal(si[1], SI[1])
    assert np.array_equal(raw, raw_r), np.flatnonzero(raw != raw_r)[:10]
    assert np.array_equal(split, split_r)
    assert len(np.unique(raw)) > 1  # the criterion sets more than one level
