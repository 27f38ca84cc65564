"""Radial-return plasticity in the CPU restatement (no counterpart in the reference, whose
plastic step is only prototyped): the yield surface is not exceeded after a step, and a
yield stress no cell reaches gives the hyperelastic (reference) bits."""
import numpy as np
import pytest

from plastic_case import YIELD, sheared_block, von_mises

from oracle import pyoracle


@pytest.mark.parametrize("flux_form", [0, 1])
def test_yield_surface_not_exceeded(flux_form, oracle_lib):
    _, F, S, solid, m5, dt = sheared_block()
    om = pyoracle.OracleMesh(F.geometry())
    m5 = dict(m5, flux_form=flux_form)
    elastic = pyoracle.m5_advance(om, S.T, dt, 2, m5).T
    plastic = pyoracle.m5_advance(om, S.T, dt, 2, dict(m5, **{"yield": [YIELD, 0.0, 0.0]})).T
    assert von_mises(elastic, m5)[solid].max() > 2.0 * YIELD  # the case yields
    assert von_mises(plastic, m5)[solid].max() <= YIELD * (1.0 + 1e-9)
    # the return keeps each material's partial density, volume fraction and alpha rho e of
    # the cell it acts on; only the deformation tensor and what the flux makes of it change
    assert np.isfinite(plastic).all()


def test_unreached_yield_stress_gives_the_hyperelastic_bits(oracle_lib):
    _, F, S, _, m5, dt = sheared_block()
    om = pyoracle.OracleMesh(F.geometry())
    a = pyoracle.m5_advance(om, S.T, dt, 2, m5)
    b = pyoracle.m5_advance(om, S.T, dt, 2, dict(m5, **{"yield": [1e30, 0.0, 0.0]}))
    assert np.array_equal(a, b)
