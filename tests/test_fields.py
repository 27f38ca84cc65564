"""Derived model-5 fields (density, mixture pressure, volume fraction, von Mises stress) used
by the FP32-form error report: checked against states built from known primitives."""
import numpy as np

from forestfv_public_gb300.fields import error_report, primitives
from forestfv_public_gb300.workloads import BUBBLE, mixture_state


def test_mixture_state_pressure_roundtrip():
    a_gas = np.array([1e-6, 0.3, 0.5, 0.9, 1.0 - 1e-6])
    S = mixture_state(BUBBLE, a_gas)
    pr = primitives(S, BUBBLE["gamma"], BUBBLE["pinf"], BUBBLE["mu"], BUBBLE["amin"])
    a1 = np.clip(a_gas, 1e-6, 1 - 1e-6)
    p_expect = (1 - a1) * BUBBLE["p"][0] + a1 * BUBBLE["p"][1]
    assert np.allclose(pr["p"], p_expect, rtol=1e-9)
    assert np.allclose(pr["rho"], (1 - a1) * 1000.0 + a1 * 1.0)
    assert np.allclose(pr["vm"], 0.0, atol=1e-6)


def solid_state(A, p=5e6, gamma=3.5, pinf=3.2e10, mu=2.6e10, rho=2700.0):
    """One-material solid cell in a 2-material layout (second material at 1e-6)."""
    N = 2
    S = np.zeros((3 * N + 12, 1))
    a = np.array([1.0 - 1e-6, 1e-6])
    S[0, 0], S[1, 0] = a[0] * rho, a[1] * 1.0
    G = A @ A.T
    d = np.linalg.det(G)
    g13 = d ** (1 / 3)
    M = G - g13 * np.eye(3)
    e_el = mu / (4 * d ** (1 / 6)) * np.trace(M @ M)
    S[2 * N + 3, 0] = a[0] * (p + gamma * pinf) / (gamma - 1) + e_el
    S[2 * N + 4, 0] = a[1] * (p + 1.4 * 0.0) / 0.4
    S[N + 3, 0] = S[2 * N + 3, 0] + S[2 * N + 4, 0]
    S[N + 4, 0] = a[0]
    S[3 * N + 3:3 * N + 12, 0] = A.reshape(-1)
    return S, (gamma, 1.4), (pinf, 0.0), (mu, 0.0)


def test_solid_stress_matches_direct_formula():
    A = np.array([[1.0, 0.01, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    S, ga, pi, mu = solid_state(A)
    pr = primitives(S, ga, pi, mu)
    G = A @ A.T
    d = np.linalg.det(G)
    dev = G @ G - np.trace(G @ G) / 3 * np.eye(3) - d ** (1 / 3) * (G - np.trace(G) / 3 * np.eye(3))
    sig = -(1 - 1e-6) * 5e6 * np.eye(3) - 1e-6 * 5e6 * np.eye(3) - mu[0] / d ** (1 / 6) * dev
    s = sig - np.trace(sig) / 3 * np.eye(3)
    vm = np.sqrt(1.5 * np.sum(s * s))
    assert np.isclose(pr["p"][0], 5e6, rtol=1e-6)
    assert np.isclose(pr["vm"][0], vm, rtol=1e-9)
    assert vm > 1e8  # 1 % shear of a 26 GPa shear-modulus solid


def test_error_report_keys_and_zero():
    S = mixture_state(BUBBLE, np.linspace(0, 1, 7))
    rep = error_report(S, S, BUBBLE["gamma"], BUBBLE["pinf"], BUBBLE["mu"])
    for k in ("rho", "p", "alpha"):
        assert rep[k]["rel_l1"] == 0.0 and rep[k]["rel_linf"] == 0.0


def test_to_uniform_paints_leaves(built_lib):
    from forestfv_public_gb300 import Mesh
    from forestfv_public_gb300.fields import to_uniform
    from forestfv_public_gb300.workloads import refine_to_target
    leaves = refine_to_target((2, 2, 2), 2, 4,
                              lambda c, h: np.where(c[:, 0] < 0.25, 4, np.where(c[:, 0] < 0.5, 3, 2)))
    m = Mesh((2, 2, 2), leaves)
    x = m.centroids()
    U = to_uniform(m, x.T.copy(), 4)
    assert U.shape == (3, 16, 16, 16)
    # every fine cell holds the centroid of the leaf that covers it
    fine = (np.stack(np.meshgrid(*[np.arange(16)] * 3, indexing="ij"), -1) + 0.5) / 16
    hl = 0.5 / (1 << (np.where(fine[..., 0] < 0.25, 4, np.where(fine[..., 0] < 0.5, 3, 2)) - 1))
    exp = (np.floor(fine / hl[..., None]) + 0.5) * hl[..., None]
    assert np.allclose(np.moveaxis(U, 0, -1), exp)
