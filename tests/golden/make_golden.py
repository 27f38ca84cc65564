"""Generate the golden fixtures under tests/golden/ by running the reference solver's own
C code (built single-rank into oracle/_ref by oracle/ref/Makefile) on synthetic cases.

Each fixture holds the case parameters, the reference's leaf list (tree index, level,
child-index path), its initial and final conserved state, its loop time, and -- for the
small cases -- its per-leaf geometry (neighbours, areas, normals, distances, volume), so
that the CPU restatement, the face-table builder and the CUDA path can be checked
against the reference on a machine where the reference is not available.

Usage: python tests/golden/make_golden.py [fixture names]
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refcase as rc  # noqa: E402

SOD = "split 0 0.5 1 0 0 0 1 0.125 0 0 0 0.1"

# name -> (Case, keep geometry)
CASES = {
    "m0_sod_uniform": (rc.Case(trees=(4, 4, 4), level=2, steps=20, dt=0.002, ic=SOD), True),
    "m0_sphere_amr": (rc.Case(trees=(2, 2, 2), level=3, steps=10, dt=0.001,
                              refine="sphere 0.5 0.5 0.5 0.3 4 3",
                              ic="sphere 0.5 0.5 0.5 0.2 1 0 0 0 1 0.125 0 0 0 0.1"), True),
    "m0_wave_box_mixedbc": (rc.Case(trees=(4, 4, 4), level=2, steps=10, dt=0.001,
                                    refine="box 0.1 0.2 0.3 0.6 0.7 0.9 4 2",
                                    bc=(2, 4, 2, 4, 1, 2), ic="wave 1 0.1 -0.2 0.3 1 0.2 1 2 1"),
                            True),
    "m0_wave_order1_rk3_reflective": (rc.Case(trees=(4, 4, 4), level=2, steps=10, dt=0.001,
                                              rk_steps=3, order=1, bc=(4,) * 6,
                                              ic="wave 1 0.1 -0.2 0.3 1 0.2 1 2 1"), True),
    "m0_stiff_rk4_allbc": (rc.Case(trees=(4, 4, 4), level=2, steps=10, dt=0.0005, rk_steps=4,
                                   gamma=4.4, pinf=6.0, bc=(1, 2, 3, 4, 1, 2),
                                   ic="wave 1 0.1 -0.2 0.3 20 0.2 1 2 1"), True),
    "m0_blast_amr_deep": (rc.Case(trees=(2, 2, 2), level=2, steps=8, dt=0.0005,
                                  refine="sphere 0.3 0.6 0.4 0.35 5 2",
                                  ic="sphere 0.3 0.6 0.4 0.2 1 0.5 -0.3 0.2 10 1 0 0 0 1"), True),
}


WALL = dict(avf_lim=0.5, prelax=3, amin=1e-6, pinf=[3.2e10, 6e8, 0.0], gamma=[3.5, 4.4, 1.4],
            mu=[2.6e10, 0.0, 0.0], rho0=[2700.0, 1000.0, 1.0], p0=[5e6, 5e6, 1e5])
WALL_IC = "m5 1 2 below 2 0.25 0 sphere 0.5 0.5 0.6 0.15 2"

M5_CASES = {
    # liquid (stiffened gas) with a gas sphere, sharp interface, iterative relaxation
    "m5_bubble_prelax3": rc.Case(trees=(2, 2, 2), level=3, steps=3, dt=1e-7, model=5,
                                 m5=dict(avf_lim=1.0, prelax=3, amin=1e-6, pinf=[6e8, 0.0],
                                         gamma=[4.4, 1.4], mu=[0.0, 0.0], rho0=[1000.0, 1.0],
                                         p0=[5e6, 1e5]),
                                 ic="m5 0 1 sphere 0.5 0.5 0.5 0.2 1"),
    # two mild materials, closed-form two-material relaxation
    "m5_mild_prelax1": rc.Case(trees=(2, 2, 2), level=3, steps=3, dt=1e-3, model=5,
                               m5=dict(avf_lim=1.0, prelax=1, amin=1e-6, pinf=[1.0, 0.0],
                                       gamma=[2.0, 1.4], mu=[0.0, 0.0], rho0=[2.0, 1.0],
                                       p0=[2.0, 1.0]),
                               ic="m5 0 1 sphere 0.5 0.5 0.5 0.2 1"),
    # hyperelastic solid below z = 0.25, liquid, gas bubble; a mixture slab whose solid
    # fraction crosses AVF_LIM exercises the ghost-fluid fluxes and both velocity fixes
    "m5_wall_gfm": rc.Case(trees=(2, 2, 2), level=3, steps=4, dt=1e-6, model=5,
                           m5=dict(WALL, mix="2 0.25 0.375 0 0.4999999 1 5e6 0 0 -50"),
                           ic=WALL_IC),
    # the same on a 2:1 mesh refined around the bubble and wall
    "m5_wall_amr": rc.Case(trees=(2, 2, 2), level=3, steps=3, dt=2e-8, model=5, m5=dict(WALL),
                           refine="sphere 0.5 0.5 0.4 0.3 4 3", ic=WALL_IC),
    "m5_wall_rk3_order1": rc.Case(trees=(2, 2, 2), level=3, steps=3, dt=2e-8, model=5,
                                  m5=dict(WALL), rk_steps=3, order=1, ic=WALL_IC),
    # symmetry planes (bc 1, m5_hllc.c:56-85) on three sides of a refined mesh with the
    # moving mixture slab, the other sides transmissive or reflective
    "m5_wall_symmetry": rc.Case(trees=(2, 2, 2), level=3, steps=4, dt=2e-7, model=5,
                                m5=dict(WALL, mix="2 0.25 0.375 0 0.4999999 1 5e6 0 0 -50"),
                                refine="sphere 0.5 0.5 0.4 0.3 4 3", bc=(1, 2, 4, 1, 1, 2),
                                ic=WALL_IC),
}


# refinement tag passes run on the final state of every model-5 case (the reference's own
# interface_location / criterionsplt / criterionsmth): (uniform, lvl, prs, lvl, thr, rho, lvl,
# thr, vel, lvl, thr, inter0, lvl, lrs, inter1, lvl, lrs) as the reference's input file gives
# them
TAG_PASSES = (
    (1, 2, 0, 0, 0.0, 1, 5, 0.05, 0, 0, 0.0, 0, 0, 0, 0, 0, 0),
    (1, 3, 1, 5, 0.3, 1, 5, 0.5, 0, 0, 0.0, 1, 4, 2, 1, 3, 1),
    (0, 0, 1, 5, 0.01, 1, 4, 0.2, 1, 5, 0.9, 1, 5, 1, 0, 0, 0),
    (1, 1, 1, 4, 0.02, 0, 0, 0.0, 0, 0, 0.0, 1, 5, 3, 0, 0, 0),
)


# the reference's own restart file (restart_save.c) of the final state of these cases
RESTART = ("m0_sphere_amr", "m5_wall_amr")

# the reference's meshadaptation on the final state of these cases (same criterion order)
ADAPT = {
    "m5_bubble_prelax3": (1, 2, 0, 0, 0.0, 1, 5, 0.05, 0, 0, 0.0, 0, 0, 0, 0, 0, 0),
    "m5_mild_prelax1": (1, 2, 1, 4, 0.2, 1, 4, 0.1, 0, 0, 0.0, 1, 4, 1, 0, 0, 0),
    "m5_wall_amr": (1, 2, 1, 4, 0.2, 1, 4, 0.1, 0, 0, 0.0, 1, 4, 1, 0, 0, 0),
}


def config1_case() -> rc.Case:
    """Plain-method Sod problem of the 32^3 uniform forest: 4^3 trees at level 4, ideal
    gas, transmissive, MUSCL-HLLC, RK_STEPS 2, 100 steps.  The reference has no CFL
    logic (DT is an input, inputset.c:69): dt is CFL 0.4 on the initial state,
    0.4 * h / max(|u| + c) with h = 1/32 and c = sqrt(1.4) on the left state."""
    h = 1.0 / 32.0
    dt = 0.4 * h / np.sqrt(1.4)
    return rc.Case(trees=(4, 4, 4), level=4, steps=100, dt=float(dt), ic=SOD)


def save(name: str, c: rc.Case, keep_geom: bool) -> None:
    init, final, _ = rc.run_case(c)
    d = dict(
        ntrees=np.array(c.trees, np.int32), bc_sides=np.array(c.bc, np.int32),
        steps=np.int32(c.steps), dt=np.float64(c.dt), rk_steps=np.int32(c.rk_steps),
        order=np.int32(c.order), gamma=np.float64(c.gamma), pinf=np.float64(c.pinf),
        root=final.root, level=final.level, adrs=final.adrs.astype(np.int8),
        S_init=init.S, S_final=final.S, ref_loop_seconds=np.float64(final.loop_seconds),
        model=np.int32(c.model),
    )
    if c.model == 5:
        for key in ("avf_lim", "prelax", "amin", "pinf", "gamma", "mu"):
            d["m5_" + key] = np.asarray(c.m5[key])
    if final.tags is not None:
        d["tag_params"] = np.asarray(c.tags, dtype=np.float64)
        d["tags"] = final.tags.astype(np.int8)
    if final.restart_text is not None:
        d["restart_text"] = np.frombuffer(final.restart_text.encode("ascii"), dtype=np.uint8)
    if final.adapted is not None:
        a = final.adapted
        d.update(adapt_params=np.asarray(c.adapt, dtype=np.float64), adapt_root=a.root,
                 adapt_level=a.level, adapt_adrs=a.adrs.astype(np.int8), adapt_S=a.S)
    if keep_geom:
        d.update(bc=final.bc.astype(np.int8), nn=final.nneig.astype(np.int8),
                 neigfc=final.neigfc.astype(np.int8), nb=final.nb, area=final.area,
                 nrm=final.normals.astype(np.int8), dist_cf=final.dist_cf,
                 dist_cc=final.dist_cc, vol=final.vol, xc=final.xc)
        assert np.array_equal(d["nrm"].astype(np.float64), final.normals)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print(f"{name}: {final.n} leaves, {c.steps} steps, reference loop {final.loop_seconds:.3f} s")


def main() -> None:
    if not rc.build_ref():
        raise SystemExit("reference oracle could not be built")
    only = set(sys.argv[1:])  # optional: names of the fixtures to regenerate
    for name, (c, g) in CASES.items():
        if not only or name in only:
            c.restart = name in RESTART
            save(name, c, g)
    for name, c in M5_CASES.items():
        if not only or name in only:
            c.tags = TAG_PASSES
            c.adapt = ADAPT.get(name)
            c.restart = name in RESTART
            save(name, c, True)
    if not only or "m0_config1_sod32" in only:
        save("m0_config1_sod32", config1_case(), False)


if __name__ == "__main__":
    main()
