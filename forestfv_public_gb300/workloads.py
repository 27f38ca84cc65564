"""Synthetic workloads of the benchmark configurations (meshes and initial states).

Everything is generated from fixed seeds; no external data.  Levels follow the reference:
trees are level 1, a leaf at level l has 2**(l-1) cells per tree edge.  With the 2^3-tree
unit cube used here, "level L" of the configurations (2**L cells per edge) is reference
level L.
"""
from __future__ import annotations

import numpy as np

from .mesh import Leaves, Mesh

# corner k of a child sits at (x, y, z) = (bit1(k), bit0(k), bit2(k))
_OFF = np.array([[(k >> 1) & 1, k & 1, (k >> 2) & 1] for k in range(8)], dtype=np.int64)


def refine_to_target(ntrees, lmin: int, lmax: int, target) -> Leaves:
    """Top-down octree refinement of every tree from level lmin: a cell of level l is
    split while target(centres, h) > l (vectorised over cells).  `target` must fall off
    by at most one level per two cells of the coarser level so that the result is 2:1
    balanced (ffv_mesh_build checks it)."""
    T = np.asarray(ntrees, dtype=np.int64)
    edge = 1.0 / T.max()
    e = 1 << (lmin - 1)
    g = np.stack(np.meshgrid(*[np.arange(t * e) for t in T], indexing="ij"), -1).reshape(-1, 3)
    out_g, out_l = [], []
    for l in range(lmin, lmax + 1):
        h = edge / (1 << (l - 1))
        cen = (g + 0.5) * h
        split = target(cen, h) > l if l < lmax else np.zeros(len(g), bool)
        out_g.append(g[~split])
        out_l.append(np.full((~split).sum(), l, np.int32))
        g = (2 * g[split][:, None, :] + _OFF[None, :, :]).reshape(-1, 3)
    gg = np.concatenate(out_g)
    ll = np.concatenate(out_l)
    per_tree = (1 << (ll - 1)).astype(np.int64)
    tree = gg // per_tree[:, None]
    cell = gg - tree * per_tree[:, None]
    return Leaves(tree.astype(np.int32), ll, cell.astype(np.int32))


BUBBLE = dict(gamma=(4.4, 1.4), pinf=(6e8, 0.0), rho=(1000.0, 1.0), p=(5e6, 1e5), mu=(0.0, 0.0),
              amin=1e-6)


def bubble_config2(lmin: int = 4, lmax: int = 8, band_cells: float = 22.0, seed: int = 20261203,
                   radius: float = 0.1):
    """Two-phase gas bubble collapse in liquid (the second configuration): liquid
    (stiffened gas, gamma 4.4, p_inf 6e8, rho 1000, p 5e6) around a gas sphere (gamma 1.4,
    rho 1, p 1e5) of radius 0.1 at the centre, interface smoothed over two finest cells
    with tanh in volume fraction, radius perturbed by seeded harmonics l <= 8 of relative
    amplitude 1e-3; 2^3 trees, levels lmin..lmax refined around the interface.
    Returns (Mesh, S [neq, n], params)."""
    leaves, state = bubble_config2_parts(lmin, lmax, band_cells, seed, radius)
    mesh = Mesh((2, 2, 2), leaves)
    return mesh, state(mesh.centroids()), dict(BUBBLE)


def bubble_config2_parts(lmin: int = 4, lmax: int = 8, band_cells: float = 22.0,
                         seed: int = 20261203, radius: float = 0.1):
    """bubble_config2 without the face tables: its leaves (2^3 trees) and the function
    from cell centroids to the initial state (numpy only)."""
    c0 = np.array([0.5, 0.5, 0.5])
    hmin = 0.5 / (1 << (lmax - 1))
    coeff_rng = np.random.default_rng(seed + 1)
    coef = [(l, m, coeff_rng.uniform(-1e-3, 1e-3)) for l in range(1, 9) for m in range(-l, l + 1)]

    def radius_at(x):
        d = x - c0
        r = np.linalg.norm(d, axis=1)
        theta = np.arccos(np.clip(d[:, 2] / np.maximum(r, 1e-300), -1, 1))
        phi = np.arctan2(d[:, 1], d[:, 0])
        from scipy.special import sph_harm_y
        s = np.zeros_like(r)
        for l, m, a in coef:
            y = sph_harm_y(l, abs(m), theta, phi)
            yr = np.sqrt(2) * (y.imag if m < 0 else y.real) if m != 0 else y.real
            s += a * yr
        return r, radius * (1.0 + s)

    def target(cen, h):
        # the refinement band follows the unperturbed sphere (the perturbation is 1e-3 R)
        r = np.linalg.norm(cen - c0, axis=1)
        d = np.abs(r - radius) - 0.8660254 * h
        lev = lmax - np.floor(np.maximum(d, 0.0) / (band_cells * hmin * 2.0)).astype(np.int64)
        return np.maximum(lev, lmin)

    def state(x):
        w = 2.0 * hmin
        r = np.linalg.norm(x - c0, axis=1)
        R = np.full_like(r, radius)
        near = np.abs(r - radius) < 20.0 * w  # the tanh profile is saturated beyond this
        r[near], R[near] = radius_at(x[near])
        a_gas = 0.5 * (1.0 - np.tanh((r - R) / w))
        return mixture_state(BUBBLE, a_gas)

    return refine_to_target((2, 2, 2), lmin, lmax, target), state


def mixture_state(mat: dict, a_gas: np.ndarray) -> np.ndarray:
    """Two-material state [neq=18, n] at rest: material 0 liquid, 1 gas, each at its own
    initial pressure weighted by volume fraction (pressure equilibrium within a cell)."""
    amin = mat["amin"]
    a1 = np.clip(a_gas, amin, 1.0 - amin)
    a0 = 1.0 - a1
    p = a0 * mat["p"][0] + a1 * mat["p"][1]
    n = len(a_gas)
    N = 2
    S = np.zeros((3 * N + 12, n))
    E = np.zeros(n)
    for k, a in enumerate((a0, a1)):
        S[k] = a * mat["rho"][k]
        are = a * (p + mat["gamma"][k] * mat["pinf"][k]) / (mat["gamma"][k] - 1.0)
        S[2 * N + 3 + k] = are
        E += are
    S[N + 3] = E
    S[N + 4] = a0
    return S


WALL = dict(gamma=(3.5, 4.4, 1.4), pinf=(3.2e10, 6e8, 0.0), rho=(2700.0, 1000.0, 1.0),
            p=(5e6, 5e6, 1e5), mu=(2.6e10, 0.0, 0.0), amin=1e-6, avf_lim=0.5,
            yield_stress=(3e8, 0.0, 0.0))


def bubble_wall_config3(lmin: int = 4, lmax: int = 9, band_cells: float = 6.5,
                        radius: float = 0.1, standoff: float = 1.5, wall_z: float = 0.2):
    """Gas bubble collapse near a solid wall (the third configuration): the half-space
    z < wall_z is a hyperelastic solid (material 0: rho 2700, stiffened-gas gamma 3.5,
    p_inf 3.2e10, shear modulus 2.6e10), above it liquid (material 1, as in the second
    configuration) around a gas sphere (material 2) of radius 0.1 centred standoff radii
    above the wall, its interface smoothed over two finest cells with tanh in volume
    fraction; 2^3 trees, levels lmin..lmax refined around the wall plane and the bubble
    (9.9 M cells at the default sizes).  The solid cells take the reference's m5_init_S
    state (init_S.c:205-266: the cell's material at 1 - 2 AMIN, the others at AMIN,
    deformation A = I; A = 0 in fluid cells).  Returns (Mesh, S [21, n], params)."""
    leaves, state = bubble_wall_parts(lmin, lmax, band_cells, radius, standoff, wall_z)
    mesh = Mesh((2, 2, 2), leaves)
    return mesh, state(mesh.centroids()), dict(WALL)


def bubble_wall_parts(lmin: int = 4, lmax: int = 9, band_cells: float = 6.5,
                      radius: float = 0.1, standoff: float = 1.5, wall_z: float = 0.2):
    """bubble_wall_config3 without the face tables: its leaves (2^3 trees) and the
    function from cell centroids to the initial state (numpy only)."""
    c0 = np.array([0.5, 0.5, wall_z + standoff * radius])
    hmin = 0.5 / (1 << (lmax - 1))

    def target(cen, h):
        r = np.linalg.norm(cen - c0, axis=1)
        d = np.minimum(np.abs(r - radius), np.abs(cen[:, 2] - wall_z)) - 0.8660254 * h
        lev = lmax - np.floor(np.maximum(d, 0.0) / (band_cells * hmin * 2.0)).astype(np.int64)
        return np.maximum(lev, lmin)

    def state(x):
        r = np.linalg.norm(x - c0, axis=1)
        a_gas = 0.5 * (1.0 - np.tanh((r - radius) / (2.0 * hmin)))
        return wall_state(WALL, x[:, 2] < wall_z, a_gas)

    return refine_to_target((2, 2, 2), lmin, lmax, target), state


def wall_state(mat: dict, solid: np.ndarray, a_gas: np.ndarray) -> np.ndarray:
    """Three-material state [neq=21, n] at rest: material 0 solid, 1 liquid, 2 gas.  Solid
    cells: the solid at 1 - 2 AMIN at its initial pressure, A = I.  Fluid cells: the solid
    at AMIN, gas fraction a_gas (clipped to [AMIN, 1 - 2 AMIN]), the liquid the rest, at the
    volume-fraction-weighted pressure, A = 0 (no elastic energy in either)."""
    amin = mat["amin"]
    N = 3
    n = len(a_gas)
    ag = np.where(solid, amin, np.clip(a_gas, amin, 1.0 - 2.0 * amin))
    asol = np.where(solid, 1.0 - 2.0 * amin, amin)
    aliq = 1.0 - asol - ag
    alpha = (asol, aliq, ag)
    p = np.where(solid, mat["p"][0], aliq * mat["p"][1] + ag * mat["p"][2])
    S = np.zeros((3 * N + 12, n))
    E = np.zeros(n)
    for k in range(N):
        S[k] = alpha[k] * mat["rho"][k]
        are = alpha[k] * (p + mat["gamma"][k] * mat["pinf"][k]) / (mat["gamma"][k] - 1.0)
        S[2 * N + 3 + k] = are
        E += are
    S[N + 3] = E
    S[N + 4] = asol
    S[N + 5] = aliq
    for q in (0, 4, 8):
        S[3 * N + 3 + q] = np.where(solid, 1.0, 0.0)
    return S


def blast_m0(mesh: Mesh, center, radius: float, p_in: float = 10.0, p_out: float = 0.1,
             rho_in: float = 1.0, rho_out: float = 0.125, gamma: float = 1.4) -> np.ndarray:
    """Model-0 spherical blast at rest: (rho_in, p_in) inside the sphere, (rho_out, p_out)
    outside; SoA state [5, n]."""
    x = mesh.centroids()
    inside = np.linalg.norm(x - np.asarray(center), axis=1) < radius
    rho = np.where(inside, rho_in, rho_out)
    p = np.where(inside, p_in, p_out)
    S = np.zeros((5, mesh.n))
    S[0] = rho
    S[4] = p / (gamma - 1.0)
    return S


def random_blast_m0(mesh: Mesh, seed: int) -> np.ndarray:
    """A seeded blast: centre uniform in [0.3, 0.7]^3, radius in [0.08, 0.2], pressure
    ratio in [20, 200]."""
    rng = np.random.default_rng(seed)
    return blast_m0(mesh, rng.uniform(0.3, 0.7, 3), rng.uniform(0.08, 0.2),
                    p_in=0.1 * rng.uniform(20.0, 200.0))


def bubble_field_parts(lbase: int = 8, lmax: int = 10, band_cells: float = 2.0, nbubbles: int = 64,
                       rmin: float = 0.02, rmax: float = 0.05, wall_z: float = 0.2,
                       seed: int = 20261203):
    """The throughput stress test (the fifth configuration) without the face tables: a
    uniform level-lbase base mesh (2^3 trees; level 8 is 256^3 cells) holding `nbubbles`
    non-overlapping gas bubbles, radii uniform in [rmin, rmax], centres drawn by seeded
    rejection sampling in the liquid above the solid half-space z < wall_z of the wall
    configuration (at least one radius of liquid between a bubble and the wall, the domain
    boundary or another bubble), the liquid at one seeded pressure uniform in 1-10 MPa;
    refined to lmax within band_cells finest cells of every bubble surface and of the wall
    plane, one level per two cells of the coarser level away from them (2:1 balanced).
    Returns (leaves, state function of cell centroids, the bubbles as (centres, radii), the
    liquid pressure)."""
    rng = np.random.default_rng(seed)
    p_liq = float(rng.uniform(1e6, 1e7))
    centres, radii = [], []
    tries = 0
    while len(radii) < nbubbles:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place the bubbles")
        r = rng.uniform(rmin, rmax)
        c = np.array([rng.uniform(2 * r, 1 - 2 * r), rng.uniform(2 * r, 1 - 2 * r),
                      rng.uniform(wall_z + 2 * r, 1 - 2 * r)])
        if all(np.linalg.norm(c - c2) > r + r2 + max(r, r2) for c2, r2 in zip(centres, radii)):
            centres.append(c)
            radii.append(r)
    C = np.array(centres)
    R = np.array(radii)
    hmin = 0.5 / (1 << (lmax - 1))

    def surface_distance(x, chunk=1 << 20):
        d = np.abs(x[:, 2] - wall_z)
        for a in range(0, len(x), chunk):
            xa = x[a:a + chunk]
            db = np.abs(np.linalg.norm(xa[:, None, :] - C[None], axis=2) - R[None]).min(axis=1)
            d[a:a + chunk] = np.minimum(d[a:a + chunk], db)
        return d

    def target(cen, h):
        d = surface_distance(cen) - 0.8660254 * h
        lev = lmax - np.floor(np.maximum(d, 0.0) / (band_cells * hmin * 2.0)).astype(np.int64)
        return np.maximum(lev, lbase)

    mat = dict(WALL, p=(5e6, p_liq, 1e5))

    def state(x, chunk=1 << 20):
        a_gas = np.zeros(len(x))
        for a in range(0, len(x), chunk):
            xa = x[a:a + chunk]
            dist = np.linalg.norm(xa[:, None, :] - C[None], axis=2) - R[None]
            a_gas[a:a + chunk] = (0.5 * (1.0 - np.tanh(dist / (2.0 * hmin)))).max(axis=1)
        return wall_state(mat, x[:, 2] < wall_z, a_gas)

    leaves = refine_to_target((2, 2, 2), lbase, lmax, target)
    return leaves, state, (C, R), p_liq


def bubble_field_config5(lbase: int = 8, lmax: int = 10, band_cells: float = 2.0,
                         seed: int = 20261203):
    """bubble_field_parts as a mesh and state: returns (Mesh, S [21, n], params)."""
    leaves, state, _, p_liq = bubble_field_parts(lbase, lmax, band_cells, seed=seed)
    mesh = Mesh((2, 2, 2), leaves)
    return mesh, state(mesh.centroids()), dict(WALL, p=(5e6, p_liq, 1e5))
