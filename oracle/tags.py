"""The reference's refinement tags in numpy (TEST INFRASTRUCTURE).

A restatement, for model 5 on the reference-form geometry (oracle/forest.py, or a fixture's
dump), of interface_location.c:7-86 (interface layers SI), criterionsplt.c:3-140 (target
levels from the uniform level, the relative-jump gradient criteria and the layers) and
criterionsmth.c:3-58 (merge consistency and 2:1 smoothing, LEVEL + 1 passes of two
in-place sweeps in leaf order).  The cell primitives follow the reference's cell form of
m5_facevalues.c (volume fractions clamped to [AMIN/100, 1 - AMIN/100] and renormalised,
each material's stiffened-gas pressure from its internal energy less the elastic energy).

Pinned against the reference's own tag passes on the fixtures' final states
(tests/test_oracle_tags.py); the GPU's tags on the benchmark's meshes are checked against it.
"""
from __future__ import annotations

import numpy as np


def _layout(N):
    return dict(i0=0, i1=N, i2=N + 3, i3=N + 4, i4=2 * N + 3, i5=3 * N + 3)


def _neighbours(geo):
    """Per cell and face, the sub-neighbour cell indices in the reference's order."""
    nb, nn = np.asarray(geo["nb"]), np.asarray(geo["nn"])
    n = nn.shape[0]
    return [[[int(nb[c, f, q]) for q in range(int(nn[c, f]))] for f in range(6)]
            for c in range(n)]


def cell_phi(S, m5):
    """phi per cell for the first two volume fractions (interface_location.c:17-46; for two
    solids the first phi is the larger solid fraction)."""
    N = (S.shape[0] - 12) // 3
    L = _layout(N)
    lo, hi = m5["amin"] / 100.0, 1.0 - m5["amin"] / 100.0
    ac = np.zeros((2, S.shape[1]))
    for i in range(N - 1):
        a = S[L["i3"] + i].copy()
        a = np.where(a <= lo, lo, np.where(a >= hi, hi, a))
        ac[i] = a
    phi = ac - m5["avf_lim"]
    nsolids = sum(1 for q in m5["mu"][:N] if q != 0.0)
    if N > 2 and nsolids == 2 and m5["mu"][0] != 0.0:
        phi[0] = np.maximum(ac[0], ac[1]) - m5["avf_lim"]
    return phi


def interface_layers(S, geo, m5, si_max):
    """SI [2][n]: 1 where phi changes sign across a face (a cell's face loop stops after the
    first face that shows a change), then layer l next to layer l - 1 for l < si_max."""
    nbs = _neighbours(geo)
    phi = cell_phi(S, m5)
    N = (S.shape[0] - 12) // 3
    n = S.shape[1]
    SI = np.zeros((2, n), np.int32)
    for c in range(n):
        for f in range(6):
            hit = False
            for o in nbs[c][f]:
                for v in range(N - 1):
                    if phi[v, c] * phi[v, o] < 0.0:
                        SI[v, c] = 1
                        hit = True
            if hit:
                break
    for lvl in range(2, si_max):
        prev = SI.copy()
        for c in range(n):
            for f in range(6):
                hit = False
                for o in nbs[c][f]:
                    for v in range(2):
                        if prev[v, o] == lvl - 1 and SI[v, c] == 0:
                            SI[v, c] = lvl
                            hit = True
                if hit:
                    break
    return SI


def _elastic_energy(A, mu):
    """state_equation.c:269-317 per cell (0 where the deformation determinant is 0)."""
    n = A.shape[1]
    M = A.T.reshape(n, 3, 3)
    G = np.einsum("nik,njk->nij", M, M)
    Gmag = (G[:, 0, 0] * (G[:, 1, 1] * G[:, 2, 2] - G[:, 1, 2] * G[:, 2, 1])
            - G[:, 0, 1] * (G[:, 1, 0] * G[:, 2, 2] - G[:, 1, 2] * G[:, 2, 0])
            + G[:, 0, 2] * (G[:, 1, 0] * G[:, 2, 1] - G[:, 1, 1] * G[:, 2, 0]))
    out = np.zeros(n)
    ok = Gmag != 0.0
    g13 = np.abs(Gmag[ok]) ** (1.0 / 3.0)
    M1 = G[ok] - g13[:, None, None] * np.eye(3)[None]
    tr = np.einsum("nij,nji->n", M1, M1)
    out[ok] = mu / (4.0 * np.abs(Gmag[ok]) ** (1.0 / 6.0)) * tr
    return out


def cell_prims(S, m5):
    """(sum_k alpha_k p_k, rho) per cell, as the reference's cell primitives give them."""
    N = (S.shape[0] - 12) // 3
    L = _layout(N)
    lo, hi = m5["amin"] / 100.0, 1.0 - m5["amin"] / 100.0
    r = np.zeros(S.shape[1])
    for i in range(N):
        r = r + S[L["i0"] + i]
    at = []
    for i in range(N - 1):
        a = S[L["i3"] + i]
        at.append(np.where(a <= lo, lo, np.where(a >= hi, hi, a)))
    s = np.zeros(S.shape[1])
    for i in range(N - 1):
        s = s + at[i]
    over = s > hi
    dif = s - hi
    for j in range(N - 1):
        at[j] = np.where(over, at[j] - (at[j] / s) * dif, at[j])
    s = np.where(over, hi, s)
    at.append(1.0 - s)
    ssum = np.zeros(S.shape[1])
    for i in range(N - 1):
        ssum = ssum + at[i]
    avf = at[:N - 1] + [1.0 - ssum]
    p = np.zeros(S.shape[1])
    A = S[L["i5"]:L["i5"] + 9]
    for i in range(N):
        mu = m5["mu"][i]
        ael = _elastic_energy(A, mu) if mu != 0.0 else 0.0
        g, pi = m5["gamma"][i], m5["pinf"][i]
        press = ((g - 1.0) * (S[L["i4"] + i] - ael) / at[i]) - g * pi
        p = p + avf[i] * press
    return p, r


def _rel_jump(x, y):
    """|y - x| / max(|y|, |x|), 0 when both are below 1e-8 (criterionsplt.c:83-89)."""
    eps = 1.0e-8
    if abs(y) > eps or abs(x) > eps:
        return abs(y - x) / max(abs(y), abs(x))
    return 0.0


def raw_levels(S, geo, m5, t, SI):
    """criterionsplt.c:3-140: the target level per cell.  t is the reference's input order
    (uniform, lvl, prs, lvl, thr, rho, lvl, thr, vel, lvl, thr, inter0, lvl, lrs, inter1,
    lvl, lrs); lrs1 as the input gives it is added to lrs0 (m5_input.c:50)."""
    uni, lu, prs, lp, tp, rho, lr, tr, vel, lv, tv, i0, l0, lrs0, i1, l1, lrs1 = t
    lrs1 = lrs0 + lrs1
    nbs = _neighbours(geo)
    pr, rr = cell_prims(S, m5)
    n = S.shape[1]
    out = np.ones(n, np.int32)
    for c in range(n):
        level = 1
        if uni == 1:
            level = max(level, int(lu))
        if prs == 1 or rho == 1 or vel == 1:
            gp = gr = gv = 0.0
            for f in range(6):
                for o in nbs[c][f]:
                    if prs == 1:
                        gp = max(gp, _rel_jump(pr[c], pr[o]))
                    grho = 0.0
                    if rho == 1:
                        grho = _rel_jump(rr[c], rr[o])
                        gr = max(gr, grho)
                    if vel == 1:  # the reference's velocity criterion reads the density jump
                        gv = max(gv, grho)
            lt = 1
            if prs == 1 and abs(gp) >= tp:
                lt = int(lp)
            if rho == 1 and abs(gr) >= tr:
                lt = int(lr)
            if vel == 1 and abs(gv) >= tv:
                lt = int(lv)
            level = max(level, lt)
        if i0 != 0:
            for v in range(2):
                si = SI[v, c]
                if 1 <= si < lrs0:
                    level = max(level, int(l0))
                if lrs0 <= si < lrs1:
                    level = max(level, int(l1))
        out[c] = level
    return out


def smooth(level, tree_ijk, cell_ijk, geo, lmax, split):
    """criterionsmth.c:3-58: LEVEL + 1 passes of the two in-place sweeps in leaf order (a leaf
    coarsens only with all eight sibling leaves, refines by one; no leaf more than one level
    below a face neighbour)."""
    split = np.asarray(split).copy()
    n = len(level)
    kid = ((cell_ijk[:, 0] & 1) << 1) | (cell_ijk[:, 1] & 1) | ((cell_ijk[:, 2] & 1) << 2)
    group = np.full(n, -1)
    for c in range(n):
        s = c - kid[c]
        if level[c] > 1 and s >= 0 and s + 8 <= n and all(
                level[s + q] == level[c] and kid[s + q] == q
                and (tree_ijk[s + q] == tree_ijk[c]).all()
                and ((cell_ijk[s + q] >> 1) == (cell_ijk[c] >> 1)).all() for q in range(8)):
            group[c] = s
    nbs = _neighbours(geo)
    flat = [[o for f in range(6) for o in nbs[c][f]] for c in range(n)]
    for _ in range(lmax + 1):
        for c in range(n):
            lv = level[c]
            if lv > 1:
                g = group[c]
                imerge = sum(1 for q in range(g, g + 8) if split[q] < level[q]) if g >= 0 else 0
                if imerge == 8:
                    split[c] = lv - 1
                elif lv > split[c]:
                    split[c] = lv
            if lv < split[c]:
                split[c] = lv + 1
        for c in range(n):
            mx = max([1] + [split[d] for d in flat[c]])
            if mx - split[c] > 1:
                split[c] = mx - 1
    return split


def level_max(t) -> int:
    """LEVEL as inputset.c:106 and m5_input.c:53 form it from the criterion levels."""
    return int(max(t[1], t[3], t[6], t[9], t[12], t[15]))


def si_max(t) -> int:
    """ADAPT_INTER_MAX (m5_input.c:50-57)."""
    if t[11] == 1 and t[14] == 1:
        return int(t[13] + t[13] + t[16])
    if t[11] == 1:
        return int(t[13])
    return 0


def tags(S, geo, m5, t, level, tree_ijk, cell_ijk):
    """(SI [2][n], raw levels, smoothed levels) of a state S [neq][n]."""
    smax = si_max(t)
    SI = interface_layers(S, geo, m5, smax) if t[11] != 0 else np.zeros((2, S.shape[1]), np.int32)
    raw = raw_levels(S, geo, m5, t, SI)
    return SI, raw, smooth(np.asarray(level), np.asarray(tree_ijk), np.asarray(cell_ijk), geo,
                           level_max(t), raw)
