"""Radial-return plasticity on the GPU: the FP64 form against the CPU restatement (1e-12
relative L-inf per conserved variable), the yield surface respected by both forms, and an
unreached yield stress giving the hyperelastic bits."""
import numpy as np
import pytest

from plastic_case import YIELD, sheared_block, von_mises

from forestfv_public_gb300 import Mesh, Solver
from oracle import pyoracle

pytestmark = pytest.mark.gpu
TOL = 1e-12


def run(lv, S, m5, dt, steps, precision, flux_form, yield_stress):
    mesh = Mesh((2, 2, 2), lv)
    s = Solver(model=5, order=2, rk_steps=2, gamma=m5["gamma"], pinf=m5["pinf"], mu=m5["mu"],
               amin=m5["amin"], avf_lim=m5["avf_lim"], prelax=3, precision=precision,
               flux_form=flux_form, yield_stress=yield_stress)
    s.set_mesh(mesh)
    s.upload_state(np.ascontiguousarray(S))
    s.step(dt, steps)
    out = s.download_state()
    s.close()
    return out


@pytest.mark.parametrize("flux_form", [0, 1])
def test_fp64_plastic_matches_oracle(flux_form, built_lib, oracle_lib):
    lv, F, S, solid, m5, dt = sheared_block()
    y = [YIELD, 0.0, 0.0]
    out = run(lv, S, m5, dt, 2, 0, flux_form, y)
    ref = pyoracle.m5_advance(pyoracle.OracleMesh(F.geometry()), S.T, dt, 2,
                              dict(m5, flux_form=flux_form, **{"yield": y})).T
    scale = np.maximum(np.abs(ref).max(axis=1), 1e-300)
    err = np.abs(out - ref).max(axis=1) / scale
    assert (err <= TOL).all(), (err.max(), int(err.argmax()))
    assert von_mises(out, m5)[solid].max() <= YIELD * (1.0 + 1e-9)


def test_fp32_form_respects_the_yield_surface(built_lib):
    lv, _, S, solid, m5, dt = sheared_block()
    out = run(lv, S, m5, dt, 2, 1, 1, [YIELD, 0.0, 0.0])
    assert von_mises(out, m5)[solid].max() <= YIELD * (1.0 + 1e-9)


@pytest.mark.parametrize("precision", [0, 1])
def test_unreached_yield_stress_gives_the_hyperelastic_bits(precision, built_lib):
    lv, _, S, _, m5, dt = sheared_block()
    a = run(lv, S, m5, dt, 2, precision, 1, None)
    b = run(lv, S, m5, dt, 2, precision, 1, [1e30, 0.0, 0.0])
    assert np.array_equal(a, b)
