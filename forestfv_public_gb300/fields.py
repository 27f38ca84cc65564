"""Derived fields of a model-5 state and the error report of the FP32-flux form.

The primitive fields follow the reference's equation of state (state_equation.c:143-317,
m5_facercnstr.c:151): each material's pressure from the stiffened-gas law
p_k = (gamma_k - 1)(alpha rho e_k - e_el) / alpha_k - gamma_k p_inf_k, the mixture pressure
sum_k alpha_k p_k, and the Cauchy stress sum_k sigma_k with
sigma_k = -alpha_k p_k I - mu_k |G|^(-1/6) (G^2 - tr(G^2)/3 I - |G|^(1/3) (G - tr G/3 I)),
G = A A^T.  All in float64 numpy, on the host.
"""
from __future__ import annotations

import numpy as np


def _layout(N: int):
    return dict(i0=0, i1=N, i2=N + 3, i3=N + 4, i4=2 * N + 3, i5=3 * N + 3)


def primitives(S: np.ndarray, gamma, pinf, mu, amin: float = 1e-6) -> dict:
    """S: SoA state [neq, n] of model 5 with N = (neq - 12) / 3 materials.  Returns
    density, mixture pressure, each material's volume fraction and the von Mises
    equivalent of the mixture stress."""
    neq, n = S.shape
    N = (neq - 12) // 3
    L = _layout(N)
    gamma = np.asarray(gamma[:N], np.float64)
    pinf = np.asarray(pinf[:N], np.float64)
    mu = np.asarray(mu[:N] if mu is not None else np.zeros(N), np.float64)
    rho = S[L["i0"]:L["i0"] + N].sum(axis=0)
    lo, hi = amin / 100.0, 1.0 - amin / 100.0
    a = np.clip(S[L["i3"]:L["i3"] + N - 1], lo, hi)
    alpha = np.vstack([a, 1.0 - a.sum(axis=0)])
    A = S[L["i5"]:L["i5"] + 9].T.reshape(n, 3, 3)
    G = A @ A.transpose(0, 2, 1)
    detG = np.linalg.det(G)
    g13 = np.cbrt(np.abs(detG))
    I = np.eye(3)[None]
    trG = np.trace(G, axis1=1, axis2=2)
    G2 = G @ G
    trG2 = np.trace(G2, axis1=1, axis2=2)
    M = G - g13[:, None, None] * I
    trM2 = np.einsum("nij,nji->n", M, M)
    with np.errstate(divide="ignore", invalid="ignore"):
        g16 = np.where(detG != 0.0, np.abs(detG) ** (1.0 / 6.0), 1.0)
    p_k = np.zeros((N, n))
    sigma = np.zeros((n, 3, 3))
    dev = G2 - trG2[:, None, None] / 3.0 * I - g13[:, None, None] * (G - trG[:, None, None] / 3.0 * I)
    for k in range(N):
        e_el = np.where(detG != 0.0, mu[k] / (4.0 * g16) * trM2, 0.0) if mu[k] != 0.0 else 0.0
        p_k[k] = (gamma[k] - 1.0) * (S[L["i4"] + k] - e_el) / alpha[k] - gamma[k] * pinf[k]
        sigma -= (alpha[k] * p_k[k])[:, None, None] * I
        if mu[k] != 0.0:
            sigma -= np.where(detG != 0.0, mu[k] / g16, 0.0)[:, None, None] * dev
    p = (alpha * p_k).sum(axis=0)
    s = sigma - np.trace(sigma, axis1=1, axis2=2)[:, None, None] / 3.0 * I
    vm = np.sqrt(1.5 * np.einsum("nij,nij->n", s, s))
    return dict(rho=rho, p=p, alpha=alpha, vm=vm)


def error_report(S_test: np.ndarray, S_ref: np.ndarray, gamma, pinf, mu, amin: float = 1e-6,
                 solid: int | None = None) -> dict:
    """Relative L1 (sum |a - b| / sum |b|) and relative L-inf (max |a - b| / max |b|) of
    density, pressure and the first volume fraction, and the relative error of the peak
    wall stress (maximum von Mises stress over the cells whose solid fraction exceeds 0.5;
    solid = index of the solid material, None when there is none)."""
    a = primitives(S_test, gamma, pinf, mu, amin)
    b = primitives(S_ref, gamma, pinf, mu, amin)
    out = {}
    for key, x, y in (("rho", a["rho"], b["rho"]), ("p", a["p"], b["p"]),
                      ("alpha", a["alpha"][0], b["alpha"][0])):
        d = np.abs(x - y)
        out[key] = {"rel_l1": float(d.sum() / max(np.abs(y).sum(), 1e-300)),
                    "rel_linf": float(d.max() / max(np.abs(y).max(), 1e-300))}
    if solid is not None:
        mask = b["alpha"][solid] > 0.5
        if mask.any():
            pa, pb = float(a["vm"][mask].max()), float(b["vm"][mask].max())
            out["peak_wall_stress"] = {"test": pa, "ref": pb,
                                       "rel_err": abs(pa - pb) / max(abs(pb), 1e-300)}
    return out


def to_uniform(mesh, F: np.ndarray, level: int) -> np.ndarray:
    """Cell values F [..., n] of an adaptive mesh painted onto the uniform grid of `level`
    (every leaf at or below that level covers 8^(level - l) fine cells): [..., X, Y, Z].
    Fields of two runs on different meshes are compared on this grid."""
    T = np.asarray(mesh.ntrees)
    e = 1 << (level - 1)
    out = np.zeros(F.shape[:-1] + tuple(int(t) * e for t in T), dtype=F.dtype)
    for l in np.unique(mesh.level):
        idx = np.flatnonzero(mesh.level == l)
        r = 1 << (level - int(l))
        if r < 1:
            raise ValueError("mesh finer than the target grid")
        g = (mesh.tree_ijk[idx].astype(np.int64) * (1 << (int(l) - 1)) + mesh.cell_ijk[idx]) * r
        o = np.arange(r)
        ox, oy, oz = np.meshgrid(o, o, o, indexing="ij")
        X = (g[:, 0, None] + ox.ravel()[None]).ravel()
        Y = (g[:, 1, None] + oy.ravel()[None]).ravel()
        Z = (g[:, 2, None] + oz.ravel()[None]).ravel()
        vals = np.repeat(F[..., idx], r ** 3, axis=-1)
        out[..., X, Y, Z] = vals
    return out


def same_leaves(ma, mb) -> bool:
    return (ma.n == mb.n and np.array_equal(ma.level, mb.level)
            and np.array_equal(ma.tree_ijk, mb.tree_ijk) and np.array_equal(ma.cell_ijk, mb.cell_ijk))


def error_report_meshes(ma, Sa, mb, Sb, gamma, pinf, mu, amin: float = 1e-6,
                        solid: int | None = None) -> dict:
    """error_report of run a against run b when their meshes may differ: cell by cell on
    identical leaves, otherwise on the uniform grid of the finest level of either mesh
    (each leaf's density, pressure, volume fraction and von Mises stress painted over the
    fine cells it covers; float32)."""
    if same_leaves(ma, mb):
        out = error_report(Sa, Sb, gamma, pinf, mu, amin, solid)
        out["compared_on"] = "identical leaves"
        return out
    lev = int(max(ma.level.max(), mb.level.max()))
    pa = primitives(Sa, gamma, pinf, mu, amin)
    pb = primitives(Sb, gamma, pinf, mu, amin)
    out = {"compared_on": f"uniform grid of level {lev}"}
    for key, fa, fb in (("rho", pa["rho"], pb["rho"]), ("p", pa["p"], pb["p"]),
                        ("alpha", pa["alpha"][0], pb["alpha"][0])):
        x = to_uniform(ma, fa.astype(np.float32), lev)
        y = to_uniform(mb, fb.astype(np.float32), lev)
        d = np.abs(x.astype(np.float64) - y)
        out[key] = {"rel_l1": float(d.sum() / max(np.abs(y).astype(np.float64).sum(), 1e-300)),
                    "rel_linf": float(d.max() / max(float(np.abs(y).max()), 1e-300))}
        del x, y, d
    if solid is not None:
        ka, kb = pa["alpha"][solid] > 0.5, pb["alpha"][solid] > 0.5
        if ka.any() and kb.any():
            va, vb = float(pa["vm"][ka].max()), float(pb["vm"][kb].max())
            out["peak_wall_stress"] = {"test": va, "ref": vb, "rel_err": abs(va - vb) / max(abs(vb), 1e-300)}
    return out
