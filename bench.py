#!/usr/bin/env python3
"""Throughput benchmark of the explicit FV step (cell-updates per second).

Default workload (--workload config3): gas-bubble collapse near an elastoplastic wall -- the
half-space z < 0.2 a solid (rho 2700, stiffened-gas gamma 3.5, p_inf 3.2e10, shear modulus
2.6e10, von Mises yield stress 3e8 Pa with a J2 radial return), above it liquid (gamma 4.4,
p_inf 6e8, rho 1000, p 5e6) around a gas sphere (gamma 1.4, rho 1, p 1e5) of radius 0.1 at
1.5 radii above the wall with a tanh interface over two finest cells; 2^3 trees refined from
level 4 to level 9 around the wall and the bubble (10.1 M cells), transmissive sides; model 5
with 3 materials (NEQ 21), MUSCL-HLLC with face-state relaxation, ghost-fluid coupling at the
solid (AVF_LIM 0.5), PRELAX 3, RK_STEPS 2.  Model 5's flux is the consistent form by default
(--flux-form; include/ffv.h FFV_FLUX_CONSISTENT: the reference's star-state energy and two flux
signs made consistent with the rest of its HLLC solver), dt CFL 0.1 on the solid's sound
speed at the finest cell.  Before timing, the reference's meshadaptation with the
configuration's criteria (relative density jump, interface layers) adapts the mesh (9.5 M
cells), and every timed loop starts from that mesh and state.

One benchmark step is one time step (all RK stages) over the whole mesh; one cell-update
is one cell advanced one time step.

  value      the metric's form: the FP32-flux form with learned AMR over `steps` steps of
             the time loop (network every step, the plain criterion as judge every 8 steps,
             regrids when it finds cells to refine), CUDA events on the solver's stream
             around the loop (judges and regrids included); state resident in HBM
  accuracy_gate  the metric's condition at the timed step count (relative L1 of density and
             the peak wall stress error, each <= 1e-4): the FP32-flux form against the FP64
             form, the headline run against the comparator, and the medium wall mesh whose wall
             is loaded within the window; pass/fail per quantity
  plain_fp64_amr  the comparator: plain FP64 with the reference's AMR (meshadaptation
             every 8 steps) over the same steps
  plain_fp64_form  plain FP64 steps alone (graph-launched, events around every step)
  fp32_flux_form / reference_flux_form  the FP32-flux form alone, its error growth against
             the FP64 form, in the consistent form and with the reference's own flux (the
             latter at CFL 0.01, where the reference's scheme runs at all)
  e2e        the learned loop through the public API with host buffers: every step
             uploads the state from pinned host memory and downloads it after
  roofline   the dominant kernel's algorithmic bytes per launch over its mean duration,
             per-kernel CUDA events on the solver's stream (ffv_profile_stage)
  cpu_baseline  the oracle's C restatement of the reference algorithm on all host cores, on
             contiguous Morton ranges of the same mesh (generated in numpy; no library of the
             product mapped)

`--workload config2` is the two-phase bubble without the wall (2.30 M cells), `config5` the
64-bubble stress test (40.8 M cells), `config1` the 32^3 Sod problem of model 0; `config2m` /
`config3m` / `config5m` are medium sizes.  `--impl reference` times the reference algorithm on
the host cores instead (the C restatement in oracle/, one process per core, each on its own
Morton range of the stated workload's mesh per round).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "cell-updates/s/GPU: FP32+learned-AMR vs plain FP64 at <=1e-4 rel L1 error"
UNIT = "cell-updates/s"
SOD = ((1.0, 0.0, 0.0, 0.0, 1.0), (0.125, 0.0, 0.0, 0.0, 0.1))
L2_FLUSH_BYTES = 256 << 20
C_LIQUID = float(np.sqrt(4.4 * (5e6 + 6e8) / 1000.0))


def sod_state(cent: np.ndarray, gamma: float = 1.4) -> np.ndarray:
    """Sod initial state in SoA, as the reference's m0_init_S (init_S.c:3-16) forms it."""
    left = cent[:, 0] < 0.5
    S = np.empty((5, len(cent)))
    for mask, (rho, u, v, w, p) in ((left, SOD[0]), (~left, SOD[1])):
        e_int = (p + gamma * 0.0) / (rho * (gamma - 1.0))
        S[0, mask] = rho
        S[1, mask] = rho * u
        S[2, mask] = rho * v
        S[3, mask] = rho * w
        S[4, mask] = rho * (e_int + 0.5 * (u * u + v * v + w * w))
    return S


# ------------------------------------------------------------------------------ workloads
def _bubble_solver_kwargs(p):
    return dict(model=5, order=2, rk_steps=2, gamma=p["gamma"], pinf=p["pinf"], mu=p["mu"],
                amin=p["amin"], avf_lim=1.0, prelax=3)


def _wall_solver_kwargs(p):
    """The wall configurations' solver: the solid elastoplastic with its von Mises yield
    stress (a J2 radial return after each relaxation; the reference's solid is hyperelastic)."""
    return dict(model=5, order=2, rk_steps=2, gamma=p["gamma"], pinf=p["pinf"], mu=p["mu"],
                amin=p["amin"], avf_lim=p["avf_lim"], prelax=3,
                yield_stress=p.get("yield_stress"))


C_SOLID = float(np.sqrt(3.5 * (5e6 + 3.2e10) / 2700.0))
# (lmax, refinement band in finest cells): full size, medium (profiler captures), small
WALL_SIZES = {"config3": (9, 6.5), "config3m": (7, 4.0), "config3s": (5, 2.0)}
# (lmin, lmax, band)
BUBBLE_SIZES = {"config2": (4, 8, 22.0), "config2m": (4, 7, 12.0), "config2s": (4, 6, 2.0)}
# 64-bubble stress test: (base level, finest level)
FIELD_SIZES = {"config5": (8, 10), "config5m": (6, 8), "config5s": (4, 6)}
FLUX_FORMS = {"reference": 0, "consistent": 1}
# CFL number of the wall configurations (dt on the solid's sound speed at the finest cell):
# with the consistent flux form and the radial return the medium wall mesh runs 400 steps at
# 0.1; the reference's own flux goes non-finite within ~20 steps at 0.03, so its legs take
# REFERENCE_FLUX_CFL
WALL_CFL = 0.1
REFERENCE_FLUX_CFL = 0.01
FLUX_FORM_NOTE = {
    0: "the reference's m5 flux as written (m5_star_region.c:59, m5_flux.c:20-34, 53-56)",
    1: "consistent: Rankine-Hugoniot star-state energy and m5_flux_gfm.c's momentum and "
       "deformation signs in m5_flux.c (a deviation from the reference, FFV_FLUX_CONSISTENT)"}


def workload_config(workload: str, n: int | None = None, levels=None) -> dict:
    """The static description of a workload, the same for both arms (the counts from the
    mesh as generated, before any adaptation)."""
    if n is None:
        F = cpu_case(workload)[0]
        n, levels = F.n, sorted(int(x) for x in np.unique(F.level))
    if workload == "config1":
        return {"workload": "config1 Sod 32^3, model 0, plain FP64, MUSCL-HLLC, RK2, CFL 0.4",
                "cells": n, "trees": [4, 4, 4], "level": 4, "dt": float(0.4 / 32.0 / np.sqrt(1.4)),
                "parallelism": "single GPU",
                "l2": "flushed between timed steps (256 MiB write); state 1.3 MB < L2"}
    if workload.startswith("config3"):
        lmax = WALL_SIZES[workload][0]
        size = {"config3": "", "config3m": " (medium size)", "config3s": " (small size)"}[workload]
        return {"workload": f"config3 bubble collapse near an elastoplastic wall{size} (von Mises "
                            f"yield 0.3 GPa), model 5 (3 materials), levels 4-{lmax} AMR; FP32-flux "
                            "+ learned AMR against plain FP64 + AMR; MUSCL-HLLC, ghost-fluid, "
                            "PRELAX 3, RK2",
                "cells": n, "levels": levels, "neq": 21,
                "dt": WALL_CFL * (0.5 / (1 << (lmax - 1))) / C_SOLID, "cfl": WALL_CFL,
                "cfl_speed": "solid sound speed, finest cell", "parallelism": "single GPU",
                "l2": f"state {8 * 21 * n / 1e6:.0f} MB > L2 (129 MB): no flush needed"}
    if workload.startswith("config5"):
        lbase, lmax = FIELD_SIZES[workload]
        size = {"config5": "", "config5m": " (medium size)", "config5s": " (small size)"}[workload]
        return {"workload": f"config5 throughput stress test{size}: 64 seeded gas bubbles "
                            f"(radii U(0.02, 0.05), liquid at one seeded pressure U(1, 10) MPa) above "
                            f"the solid half-space, uniform level {lbase} refined to level {lmax} "
                            "at the interfaces, model 5 (3 materials); FP32-flux + learned AMR "
                            "against plain FP64 + AMR; MUSCL-HLLC, ghost-fluid, PRELAX 3, RK2",
                "cells": n, "levels": levels, "neq": 21,
                "dt": WALL_CFL * (0.5 / (1 << (lmax - 1))) / C_SOLID, "cfl": WALL_CFL,
                "cfl_speed": "solid sound speed, finest cell", "parallelism": "single GPU",
                "l2": f"state {8 * 21 * n / 1e6:.0f} MB > L2 (129 MB): no flush needed"}
    lmin, lmax, _ = BUBBLE_SIZES[workload]
    size = {"config2": "", "config2m": " (medium size)", "config2s": " (small size)"}[workload]
    return {"workload": f"config2 bubble collapse in liquid{size}, model 5 (2 materials), levels "
                        f"{lmin}-{lmax} AMR, plain FP64 and FP32-flux forms, MUSCL-HLLC, PRELAX 3, RK2",
            "cells": n, "levels": levels, "neq": 18,
            "dt": 0.01 * (0.5 / (1 << (lmax - 1))) / C_LIQUID, "cfl": 0.01,
            "parallelism": "single GPU",
            "l2": f"state {8 * 18 * n / 1e6:.0f} MB > L2 (129 MB): no flush needed"}


def _config2(name: str):
    from forestfv_public_gb300 import workloads as W
    lmin, lmax, band = BUBBLE_SIZES[name]
    mesh, S0, p = W.bubble_config2(lmin=lmin, lmax=lmax, band_cells=band)
    cfg = workload_config(name, int(mesh.n), sorted(int(x) for x in np.unique(mesh.level)))
    alg = m5_alg_bytes(S0.shape[0], 2)
    return mesh, S0, cfg["dt"], cfg, _bubble_solver_kwargs(p), alg, False


def wl_config2(small: bool = False, medium: bool = False):
    return _config2("config2s" if small else "config2m" if medium else "config2")


def wl_config2m(small: bool = False):
    """config2 physics on a 0.36 M-cell mesh (levels 4-7): the size profiler captures use."""
    return _config2("config2s" if small else "config2m")


def wl_config1(small: bool = False):
    from forestfv_public_gb300 import Mesh, uniform_leaves
    trees, level = (4, 4, 4), 4
    mesh = Mesh(trees, uniform_leaves(trees, level))
    S0 = sod_state(mesh.centroids())
    cfg = workload_config("config1", int(mesh.n), [level])
    alg = {"m0_recon": 40 + 28 + 240, "m0_flux_rk<2>": 240 + 40 + 40 + 28 + 40}
    return mesh, S0, cfg["dt"], cfg, dict(model=0), alg, True


def _config3(name: str):
    """Bubble collapse near an elastoplastic wall (radial return at the configuration's
    yield stress), 3 materials (NEQ 21)."""
    from forestfv_public_gb300 import workloads as W
    lmax, band = WALL_SIZES[name]
    mesh, S0, p = W.bubble_wall_config3(lmax=lmax, band_cells=band)
    cfg = workload_config(name, int(mesh.n), sorted(int(x) for x in np.unique(mesh.level)))
    cfg["amr"] = {"tags": list(wall_tags(lmax)), "every": AMR_EVERY, "horizon": AMR_HORIZON,
                  "threshold": AMR_THRESHOLD, "infer_every": AMR_INFER_EVERY}
    return mesh, S0, cfg["dt"], cfg, _wall_solver_kwargs(p), m5_alg_bytes(21, 3), False


def wl_config3(small: bool = False, medium: bool = False):
    return _config3("config3s" if small else "config3m" if medium else "config3")


def wl_config3m(small: bool = False):
    """config3 physics on a 0.41 M-cell mesh (levels 4-7): the size profiler captures use."""
    return _config3("config3s" if small else "config3m")


AMR_EVERY, AMR_HORIZON, AMR_THRESHOLD = 8, 8, 0.3
# the network runs every step, as the learned-indicator configuration specifies (AdaptiveRun
# takes infer_every > 1 too: a mark predicts a refinement within AMR_HORIZON steps and the
# marks accumulate until the next regrid)
AMR_INFER_EVERY = 1
WALL_LRS = 16


def wall_tags(lmax: int) -> tuple:
    """Refinement criteria of the wall configuration in the reference's input order:
    uniform level 4, the relative density jump 0.1 and WALL_LRS interface layers, both to
    the finest level."""
    return (1, 4, 0, 0, 0.0, 1, lmax, 0.1, 0, 0, 0.0, 1, lmax, WALL_LRS, 0, 0, 0)


def m5_alg_bytes(neq: int, nmat: int) -> dict:
    """Algorithmic bytes per cell of each model-5 kernel (compulsory traffic, neighbour
    re-reads excluded).  FP32 form: the FP32 shadow state (4 neq), the 2 N critical slots in
    FP64, face records of neq + N + 1 FP32 values."""
    d = 8 * neq
    rec = 4 * (neq + nmat + 1)
    return {"m5_recon_face": d + 28 + 6 * d,
            "m5_face_flux": 6 * d + d + 28 + 6 * d + 6 * 3 * 8 + 6 * 8,
            "m5_cell_update": d + 6 * d + 6 * 3 * 8 + d + 28 + d + d + 1,
            "m5_relax_cell": d + d + 1,
            "m5f_recon_face": 4 * neq + 8 * 2 * nmat + 28 + 6 * rec,
            "m5f_face_flux": 6 * rec + 8 * 2 * nmat + 28 + 6 * 4 * neq + 6 * 3 * 4 + 6 * 8,
            "m5f_cell_update": d + 6 * 4 * neq + 6 * 3 * 4 + d + 28 + d + d + 1,
            "m5f_relax_cell": d + d + 1}


def _config5(name: str):
    """The 64-bubble throughput stress test above the solid half-space, 3 materials."""
    from forestfv_public_gb300 import workloads as W
    lbase, lmax = FIELD_SIZES[name]
    mesh, S0, p = W.bubble_field_config5(lbase=lbase, lmax=lmax)
    cfg = workload_config(name, int(mesh.n), sorted(int(x) for x in np.unique(mesh.level)))
    # uniform base level, density jump and four interface layers (the generator's band) to
    # the finest level
    cfg["amr"] = {"tags": [1, lbase, 0, 0, 0.0, 1, lmax, 0.1, 0, 0, 0.0, 1, lmax, 4, 0, 0, 0],
                  "every": AMR_EVERY, "horizon": AMR_HORIZON, "threshold": AMR_THRESHOLD,
                  "infer_every": AMR_INFER_EVERY}
    return mesh, S0, cfg["dt"], cfg, _wall_solver_kwargs(p), m5_alg_bytes(21, 3), False


def wl_config5(small: bool = False, medium: bool = False):
    return _config5("config5s" if small else "config5m" if medium else "config5")


def wl_config5m(small: bool = False):
    """config5 physics on a 1.9 M-cell mesh (levels 6-8)."""
    return _config5("config5s" if small else "config5m")


WORKLOADS = {"config2": wl_config2, "config1": wl_config1, "config2m": wl_config2m,
             "config3": wl_config3, "config3m": wl_config3m, "config5": wl_config5,
             "config5m": wl_config5m}


# ------------------------------------------------------------------------------ helpers
def max_over_ranks(t_ms: float, device) -> float:
    """The slowest rank's time: with N ranks every rank runs its own replica of the
    workload (the step does not shard here), and the whole job's rate is N replicas over
    the slowest one's time."""
    import torch
    t = torch.tensor([t_ms], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def peak_hbm() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_summary(kernel: str, cells: int, workload: str):
    """(DRAM bytes per launch, FP64-pipe % busy) of a kernel on a workload family (config2
    for config2 and config2m, ...) from the committed ncu summary (bytes per cell x cells);
    None where the kernel has no capture."""
    fam = workload[:-1] if workload.endswith("m") else workload
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for ln in open(p):
            t = ln.split()
            if len(t) >= 3 and not ln.startswith("#") and t[0] == kernel and t[1] == fam:
                return float(t[2]) * cells, (float(t[3]) if len(t) > 3 else None)
    except OSError:
        pass
    return None, None


# ------------------------------------------------------------------------ CPU legs
# The reference algorithm on the host cores: the oracle's C restatement (oracle/, the
# reference's m0/m5 step function by function) on contiguous Morton ranges of the stated
# workload's own mesh.  The mesh is generated and its reference-form geometry built in numpy
# (oracle/forest.py), so these legs map no library of the product.  A range is advanced as a
# mesh of its own (faces to cells outside it transmissive); every cell of it is a full
# cell-update of the workload's physics at its own level.


def cpu_case(workload: str):
    """(forest, initial-state function, dt, solver keywords, mesh description) of a
    workload, built in numpy only."""
    from forestfv_public_gb300 import workloads as W
    from oracle.forest import Forest
    if workload == "config1":
        from forestfv_public_gb300.mesh import uniform_leaves
        lv = uniform_leaves((4, 4, 4), 4)
        F = Forest((4, 4, 4), lv.tree_ijk, lv.level, lv.cell_ijk)
        return F, sod_state, 0.4 * (1.0 / 32.0) / np.sqrt(1.4), dict(model=0), "32^3 uniform"
    if workload.startswith("config3"):
        lmax, band = WALL_SIZES[workload]
        lv, state = W.bubble_wall_parts(lmax=lmax, band_cells=band)
        kw = _wall_solver_kwargs(W.WALL)
        dt = WALL_CFL * (0.5 / (1 << (lmax - 1))) / C_SOLID
    elif workload.startswith("config5"):
        lbase, lmax = FIELD_SIZES[workload]
        lv, state, _, _ = W.bubble_field_parts(lbase=lbase, lmax=lmax)
        kw = _wall_solver_kwargs(W.WALL)
        dt = WALL_CFL * (0.5 / (1 << (lmax - 1))) / C_SOLID
    else:
        lmin, lmax, band = BUBBLE_SIZES[workload]
        lv, state = W.bubble_config2_parts(lmin=lmin, lmax=lmax, band_cells=band)
        kw = _bubble_solver_kwargs(W.BUBBLE)
        dt = 0.01 * (0.5 / (1 << (lmax - 1))) / C_LIQUID
    F = Forest((2, 2, 2), lv.tree_ijk, lv.level, lv.cell_ijk)
    return F, state, dt, kw, f"levels {int(lv.level.min())}-{lmax}, {F.n} cells as generated"


def _cpu_advance(om, S_aos, dt, steps, kw, flux_form):
    from oracle import pyoracle
    if kw.get("model", 0) == 5:
        m5 = dict(avf_lim=kw["avf_lim"], prelax=kw["prelax"], amin=kw["amin"],
                  pinf=list(kw["pinf"]), gamma=list(kw["gamma"]), mu=list(kw["mu"]),
                  flux_form=flux_form, **{"yield": list(kw.get("yield_stress") or ())})
        return pyoracle.m5_advance(om, S_aos, dt, steps, m5)
    return pyoracle.m0_advance(om, S_aos, dt, steps)


def _cpu_range_worker(job):
    """One worker's share of a round: one untimed step of its range, then `steps` timed
    steps.  Returns (cells, steps, seconds)."""
    from oracle import pyoracle
    geo, S, dt, kw, flux_form, steps = job
    om = pyoracle.OracleMesh(geo)
    S = _cpu_advance(om, np.ascontiguousarray(S.T), dt, 1, kw, flux_form)
    t0 = time.perf_counter()
    _cpu_advance(om, S, dt, steps, kw, flux_form)
    return om.n, steps, time.perf_counter() - t0


class CpuSampler:
    """The reference algorithm timed on `cores` host processes over contiguous Morton ranges
    of a workload's mesh.  Each round gives every worker its own range (the ranges of all
    rounds spread evenly over the mesh); a worker times only its steady steps, and a round's
    rate is the sum of its workers' rates (they run at once, one per core)."""

    def __init__(self, workload: str, cores: int, flux_form: int, seconds: float = 1.0):
        from multiprocessing import get_context
        self.F, self.state, self.dt, self.kw, self.mesh_desc = cpu_case(workload)
        self.cores, self.flux_form = cores, flux_form
        self.pool = get_context("spawn").Pool(cores)
        # range size from a probe step: about `seconds` of steady work per worker and round
        probe = min(self.F.n, 4096)
        n, k, el = _cpu_range_worker(self._job(0, probe, 1))
        self.R = int(min(self.F.n, max(2048, seconds * n * k / max(el, 1e-9))))

    def _job(self, start, R, steps):
        sel = np.arange(start, start + R)
        return (self.F.geometry(sel), self.state(self.F.centroids(sel)), self.dt, self.kw,
                self.flux_form, steps)

    def round(self, index: int, rounds: int, steps: int = 1):
        """Returns (summed rate in cell-updates/s, the slowest worker's seconds)."""
        jobs = []
        for w in range(self.cores):
            i = index * self.cores + w
            c = int((i + 0.5) * self.F.n / (rounds * self.cores)) - self.R // 2
            jobs.append(self._job(min(max(c, 0), self.F.n - self.R), self.R, steps))
        res = self.pool.map(_cpu_range_worker, jobs)
        return sum(n * k / el for n, k, el in res), max(el for _, _, el in res)

    def describe(self, rounds: int, steps: int = 1) -> str:
        return (f"{self.cores} processes x {rounds} rounds; each process advances a contiguous "
                f"Morton range of {self.R} cells of the workload's mesh ({self.mesh_desc}) "
                f"by one untimed and {steps} timed time step(s) of the oracle's C restatement "
                "of the reference algorithm; ranges spread evenly over the mesh, faces leaving "
                "a range transmissive; rate = sum of the processes' rates")

    def close(self):
        self.pool.close()
        self.pool.join()


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    flux_form = FLUX_FORMS[args.flux_form]
    cfg = workload_config(args.workload)
    sampler = CpuSampler(args.workload, cores, flux_form)
    for r in range(args.warmup):
        sampler.round(r, args.warmup)
    rates, secs = [], []
    for r in range(args.steps):
        rate, el = sampler.round(r, args.steps)
        rates.append(rate)
        secs.append(el)
    sampler.close()
    value = statistics.median(rates)
    cfg["sample"] = {"cells_per_round": sampler.R * cores, "range_cells": sampler.R,
                     "processes": cores, "mesh": sampler.mesh_desc,
                     "fraction_of_mesh_per_round": sampler.R * cores / sampler.F.n}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(secs),
        "higher_is_better": True, "dtype": "f64", "data": "synthetic", "config": cfg,
        "vs_baseline": None,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sampler.describe(args.steps)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


FP32_PERTURBATION = 1e-7


def measure_fp32_form(mesh, S0, dt, kw, args, dev, fp64_solver) -> dict:
    """The FP32-flux form (precision FFV_FP32_FLUX) on the same workload: throughput with
    CUDA events on its stream, per-kernel times, and its error against the FP64 form after
    `args.steps` steps next to the FP64 form's own spread when its initial state is
    perturbed by FP32_PERTURBATION (relative, seeded): the sensitivity floor that any
    re-rounded arithmetic meets on this problem."""
    import torch

    from forestfv_public_gb300 import Solver
    from forestfv_public_gb300.fields import error_report
    s32 = Solver(device=dev.index, precision=1, **kw)
    s32.set_mesh(mesh)
    s32.upload_state(S0)
    stream = torch.cuda.ExternalStream(s32.stream_handle(), device=dev)
    s32.step(dt, args.warmup)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    torch.cuda.synchronize(dev)
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            ev[k][0].record(stream)
        s32.step_async(dt, 1)
        ev[k][1].record(stream)
    s32.sync()
    torch.cuda.synchronize(dev)
    t_ms = sum(a.elapsed_time(b) for a, b in ev)
    per_kernel = {}
    for _ in range(3):
        for irk in (1, 2):
            for name, ms in s32.profile_stage(irk, dt).items():
                per_kernel.setdefault(name, []).append(ms)
    mean_ms = {k: sum(v) / len(v) for k, v in per_kernel.items()}

    mu = kw.get("mu")
    solid = 0 if mu is not None and mu[0] != 0.0 else None
    # error growth: the FP32 form and the FP64 form from a perturbed initial state, each
    # against the FP64 form, at a few step counts (three solvers advanced side by side)
    rng = np.random.default_rng(20261203)
    Sp = S0 * (1.0 + FP32_PERTURBATION * rng.uniform(-1.0, 1.0, S0.shape))
    sper = Solver(device=dev.index, precision=0, **kw)
    sper.set_mesh(mesh)
    for s, S in ((fp64_solver, S0), (s32, S0), (sper, Sp)):
        s.upload_state(S)
    growth, done = [], 0
    for c in sorted({min(5, args.steps), min(10, args.steps), args.steps}):
        for s in (fp64_solver, s32, sper):
            s.step(dt, c - done)
        done = c
        ref = fp64_solver.download_state()
        e32 = error_report(s32.download_state(), ref, kw["gamma"], kw["pinf"], mu, kw["amin"],
                           solid)
        efl = error_report(sper.download_state(), ref, kw["gamma"], kw["pinf"], mu, kw["amin"],
                           solid)
        growth.append({"steps": c, "fp32_form": e32, "fp64_perturbed": efl})
        del ref
    sper.close()
    err, floor = growth[-1]["fp32_form"], growth[-1]["fp64_perturbed"]
    s32.close()
    return {"value": mesh.n * args.steps / (t_ms / 1e3), "unit": UNIT,
            "ms_per_step": t_ms / args.steps, "kernel_mean_ms_per_stage": mean_ms,
            "flux_form": FLUX_FORM_NOTE[kw.get("flux_form", 0)],
            "error_vs_fp64": err, "error_steps": args.steps,
            "gate": accuracy_gate(err, args.steps, kw.get("mu")),
            "fp64_sensitivity_floor": {"perturbation": FP32_PERTURBATION, **floor},
            "error_growth": growth,
            "note": "error of the FP32-flux form against the FP64 form on the same mesh after "
                    "error_steps steps, beside the FP64 form's own change when its initial state "
                    "is perturbed by 1e-7 relative (the sensitivity of the scheme itself)"}


GATE_BAR = 1e-4
# the smallest wall stress whose relative error the gate takes as it is: a strain of 1e-6
# (stress 1e-6 mu, ~16 FP32 ulps of the deformation tensor); below it the peak is rounding
# noise of a solid not yet loaded, and its error is taken relative to this scale
WALL_STRAIN_SCALE = 1e-6


def accuracy_gate(err: dict, steps: int, mu=None) -> dict:
    """The metric's accuracy condition on an error report: relative L1 error of density and
    the error of the peak wall stress, each <= 1e-4.  The wall stress error is relative to
    the larger of the FP64 peak and 1e-6 of the solid's shear modulus; the plain relative
    error is reported beside it."""
    rho = err["rho"]["rel_l1"]
    out = {"bar": GATE_BAR, "steps": steps, "rho_rel_l1": rho}
    ok = rho <= GATE_BAR
    w = err.get("peak_wall_stress")
    if w is not None:
        scale = max(abs(w["ref"]), WALL_STRAIN_SCALE * max(mu or (0.0,)))
        rel = abs(w["test"] - w["ref"]) / max(scale, 1e-300)
        out.update({"peak_wall_stress_fp64": w["ref"], "peak_wall_stress_test": w["test"],
                    "peak_wall_stress_rel_err": w["rel_err"],
                    "peak_wall_stress_err_of_scale": rel, "wall_stress_scale": scale})
        ok = ok and rel <= GATE_BAR
    out["pass"] = bool(ok)
    return out


def gate_medium(kw: dict, dev, counts=(20, 100)) -> dict:
    """The accuracy condition on the medium wall mesh (0.41 M cells, levels 4-7), where the
    wall is loaded within the first steps (peak wall stress 3e5 Pa after 20 steps): the
    FP32-flux form against the FP64 form, same mesh, same flux form."""
    from forestfv_public_gb300 import Solver
    from forestfv_public_gb300.fields import error_report
    mesh, S0, dt, _, kw_m, _, _ = wl_config3m()
    kw_m = dict(kw_m, flux_form=kw.get("flux_form", 0))
    a = Solver(device=dev.index, precision=0, **kw_m)
    b = Solver(device=dev.index, precision=1, **kw_m)
    for s in (a, b):
        s.set_mesh(mesh)
        s.upload_state(S0)
    out, done = [], 0
    try:
        for c in counts:
            a.step(dt, c - done)
            b.step(dt, c - done)
            done = c
            e = error_report(b.download_state(), a.download_state(), kw_m["gamma"], kw_m["pinf"],
                             kw_m["mu"], kw_m["amin"], 0)
            out.append(accuracy_gate(e, c, kw_m["mu"]))
    except Exception as ex:  # the reference's flux goes non-finite within ~100 steps here
        out.append({"steps": c, "error": str(ex), "pass": False})
    finally:
        a.close()
        b.close()
    return {"workload": f"config3m ({mesh.n} cells, levels 4-7)", "gates": out,
            "pass": all(g["pass"] for g in out)}


TRAIN_LMAX, TRAIN_RUNS, TRAIN_WINDOWS = 9, 3, 2  # ~9.5 M cells per snapshot: ~57 M pairs


def train_wall_indicator(kw: dict, dev, amr_cfg: dict, seed: int = 20261203):
    """The indicator of the wall configuration, trained on the GPU on seeded runs of the
    configuration's physics on levels 4-9 with standoffs U(1.0, 2.5) and bubble radii
    U(0.05, 0.15): snapshots of (features, "the criterion asks for a finer level within
    `horizon` steps") -- TRAIN_RUNS runs of TRAIN_WINDOWS snapshots, about the ~50 M pairs
    the learned-indicator configuration names -- a criterion-driven regrid between
    snapshots, then AdamW (lr 1e-3, batch 8192).  Returns the indicator and a summary."""
    import torch

    from forestfv_public_gb300 import Solver
    from forestfv_public_gb300 import workloads as W
    from forestfv_public_gb300.amr import AdaptiveRun
    from forestfv_public_gb300.indicator import Indicator, collect_window, field_norm
    t0 = time.perf_counter()
    rng = np.random.default_rng(seed)
    ind = Indicator(device=dev.index, seed=seed)
    tags_t = wall_tags(TRAIN_LMAX)
    dt_t = WALL_CFL * (0.5 / (1 << (TRAIN_LMAX - 1))) / C_SOLID
    Xs, ys, runs = [], [], 0
    for k in range(TRAIN_RUNS):
        standoff, radius = rng.uniform(1.0, 2.5), rng.uniform(0.05, 0.15)
        mesh, S0, _ = W.bubble_wall_config3(lmax=TRAIN_LMAX, band_cells=WALL_SIZES["config3"][1],
                                            radius=radius, standoff=standoff)
        s = Solver(device=dev.index, precision=1, **kw)
        s.set_mesh(mesh)
        s.upload_state(S0)
        amr = AdaptiveRun(s, tags_t)
        amr.meshadaptation()
        if k == 0:
            mean, std = field_norm([ind.fields(s).cpu().numpy()])
            ind.set_norm(mean, np.maximum(std, np.array([0.05, 0.05, 0.01, 0.01, 1.0],
                                                         np.float32)))
        for _ in range(TRAIN_WINDOWS):
            X, y = collect_window(s, ind, tags_t, dt_t, amr_cfg["horizon"])
            Xs.append(X)
            ys.append(y)
            amr.meshadaptation()
        s.close()
        runs += 1
    X, y = torch.cat(Xs), torch.cat(ys)
    losses = ind.train(X, y, steps=800, batch=8192, lr=1e-3, wd=1e-4, seed=seed)
    return ind, {"runs": runs, "pairs": int(X.shape[0]), "positive_fraction": float(y.mean()),
                 "loss_first": float(losses[:10].mean()), "loss_last": float(losses[-50:].mean()),
                 "train_steps": 800, "seconds": time.perf_counter() - t0}


def timed_amr_loop(solver, amr, dt, steps, warmup, stream, host=False):
    """Run `warmup` untimed and `steps` timed steps of an AdaptiveRun; CUDA events on the
    solver's stream bracket the timed steps (the host work of judges and regrids happens
    between them, so the events see it).  With host=True every step uploads the state from
    pinned host memory first and downloads it after (the end-to-end form).  Returns
    (seconds, cell-updates, h2d bytes, d2h bytes)."""
    import torch
    amr.run(dt, warmup)
    cu0 = amr.stats.cell_updates
    h2d = d2h = 0
    pinned = None
    if host:
        # one pinned buffer, allocated before the timed region with room for the meshes a
        # regrid makes (the state of n cells is its first neq * n doubles, [neq][n])
        pinned = torch.empty(solver.neq * (solver.mesh.n + solver.mesh.n // 2),
                             dtype=torch.float64, pin_memory=True).numpy()
        solver.download_state(out=pinned[:solver.neq * solver.mesh.n].reshape(solver.neq, -1))

    def state_buf():
        n = solver.mesh.n
        assert solver.neq * n <= pinned.shape[0], "regrid beyond the pinned buffer's headroom"
        return pinned[:solver.neq * n].reshape(solver.neq, n)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
    for _ in range(steps):
        if host:
            buf = state_buf()
            solver.upload_state(buf)
            h2d += buf.nbytes
        amr.run(dt, 1)
        if host:
            buf = state_buf()  # the step's regrid may have changed the mesh
            solver.download_state(out=buf)
            d2h += buf.nbytes
    with torch.cuda.stream(stream):
        e1.record(stream)
    solver.sync()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3, amr.stats.cell_updates - cu0, h2d, d2h


def amr_launches(solver, st, judge_launches: int) -> int:
    """Kernel launches of an AdaptiveRun's steps, judges and inferences (regrids not
    counted): launches per step x steps, judge_launches per judge, 2 per inference
    (fields, and the fused gather + tcgen05 forward + marks)."""
    return solver.launches_per_step() * st.steps + judge_launches * st.judged + 2 * st.inferences


def run_ours(args) -> None:
    import torch

    from forestfv_public_gb300 import Solver
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    mesh, S0, dt, cfg, kw, alg_bytes, flush_l2 = WORKLOADS[args.workload]()
    flux_form = FLUX_FORMS[args.flux_form]
    if kw.get("model", 0) == 5:
        kw["flux_form"] = flux_form
        cfg["flux_form"] = FLUX_FORM_NOTE[flux_form]
    amr_cfg = cfg.get("amr") if not args.no_amr else None
    solver = Solver(device=local, **kw)
    solver.set_mesh(mesh)
    solver.upload_state(S0)
    if amr_cfg is not None:
        # the timed loops start from the criterion's own mesh (the reference's meshadaptation
        # on the initial state), untimed
        from forestfv_public_gb300.amr import AdaptiveRun
        t0 = time.perf_counter()
        rounds = AdaptiveRun(solver, amr_cfg["tags"]).meshadaptation()
        mesh = solver.mesh
        S0 = solver.download_state()
        cfg["initial_adaptation"] = {"rounds": rounds, "seconds": time.perf_counter() - t0,
                                     "cells": int(mesh.n),
                                     "levels": sorted(int(x) for x in np.unique(mesh.level))}
        # the timed loops run on the adapted mesh
        cfg["cells_generated"], cfg["cells"] = cfg["cells"], int(mesh.n)
    neq = solver.neq
    stream = torch.cuda.ExternalStream(solver.stream_handle(), device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev) if flush_l2 else None

    solver.step(dt, args.warmup)  # warm-up (also builds the step graph)

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = ClockSampler()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            if flush is not None:
                flush.zero_()
            ev[k][0].record(stream)
        solver.step_async(dt, 1)
        ev[k][1].record(stream)
    solver.sync()
    torch.cuda.synchronize(dev)
    t_ms = sum(a.elapsed_time(b) for a, b in ev)
    if world > 1:
        t_ms = max_over_ranks(t_ms, dev)
    value_fp64 = world * mesh.n * args.steps / (t_ms / 1e3)

    def kernel_times(s, nprof):
        per = {}
        for _ in range(nprof):
            for irk in (1, 2):
                if flush is not None:
                    with torch.cuda.stream(stream):
                        flush.zero_()
                for name, ms in s.profile_stage(irk, dt).items():
                    per.setdefault(name, []).append(ms)
        return {k: sum(v) / len(v) for k, v in per.items()}

    def roofline_of(mean_ms, n, note):
        dom = max(mean_ms, key=mean_ms.get)
        peak, peak_kind = peak_hbm()
        alg = alg_bytes.get(dom, 0) * n
        achieved = alg / (mean_ms[dom] / 1e3) / 1e9
        step_ms = sum(mean_ms.values())
        traffic, pipe_pct = ncu_summary(dom, n, args.workload)
        return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                "fp64_pipe_busy_pct_ncu": pipe_pct,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst)",
                "kernel_mean_ms_per_stage": mean_ms,
                "kernel_share": {k: v / step_ms for k, v in mean_ms.items()},
                "alg_bytes_per_launch": alg, "note": note}

    roof64 = roofline_of(kernel_times(solver, max(3, min(args.steps, 10))), mesh.n,
                         "the FP64 kernels are FP64-pipe bound (GB300 FP64 = 1/64 FP32), "
                         "see profiles/")

    # end to end through the public API with pinned host buffers (plain FP64 form)
    host = torch.empty((neq, mesh.n), dtype=torch.float64, pin_memory=True).numpy()
    host[:] = S0
    torch.cuda.synchronize(dev)
    e2e_steps = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.upload_state(host)
        solver.step(dt, 1)
        solver.download_state(out=host)
    e2e_s = time.perf_counter() - t0
    e2e64 = {"value": world * mesh.n * e2e_steps / e2e_s, "unit": UNIT,
             "h2d_bytes_per_step": neq * 8 * mesh.n, "d2h_bytes_per_step": neq * 8 * mesh.n,
             "steps": e2e_steps}

    if rank == 0:
        cpu = None
        if world == 1 and args.cpu_rounds > 0:
            cores = os.cpu_count() or 1
            sampler = CpuSampler(args.workload, cores, flux_form)
            rates = [sampler.round(r, args.cpu_rounds)[0] for r in range(args.cpu_rounds)]
            sampler.close()
            cpu = {"value": statistics.median(rates), "unit": UNIT, "cores": cores, "kind": "port",
                   "sample": sampler.describe(args.cpu_rounds)}
        fp32 = None
        if world == 1 and kw.get("model", 0) == 5 and not args.no_fp32_form:
            fp32 = measure_fp32_form(mesh, S0, dt, kw, args, dev, solver)
            fp32["speedup_vs_fp64"] = fp32["value"] / value_fp64
        fp64_line = {"value": value_fp64, "unit": UNIT, "ms_per_step": t_ms / args.steps,
                     "e2e": e2e64, "roofline": roof64,
                     "gpu_launches": solver.launches_per_step() * args.steps}
        line = {
            "metric": METRIC, "value": value_fp64, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg, "e2e": e2e64, "roofline": roof64,
            "cpu_baseline": cpu, "gpu_launches": fp64_line["gpu_launches"],
        }
        if amr_cfg is not None and world == 1:
            line.update(measure_amr(mesh, S0, dt, kw, args, dev, amr_cfg, alg_bytes,
                                    roofline_of, kernel_times, stream))
            line["plain_fp64_form"] = fp64_line
        if fp32 is not None:
            line["fp32_flux_form"] = fp32
        if "learned_amr" in line and fp32 is not None:
            # the metric's accuracy condition at the timed step count: the FP32-flux form
            # against the FP64 form on the same mesh, and the headline run (FP32 flux +
            # learned AMR) against the comparator (FP64 + the reference's AMR)
            g_same, g_run = fp32["gate"], line["learned_amr"]["gate"]
            g_med = gate_medium(kw, dev) if args.workload == "config3" else None
            line["accuracy_gate"] = {"bar": GATE_BAR, "steps": args.steps,
                                     "fp32_vs_fp64_same_mesh": g_same,
                                     "learned_amr_vs_plain_fp64_amr": g_run,
                                     "medium_mesh_loaded_wall": g_med,
                                     "pass": bool(g_same["pass"] and g_run["pass"]
                                                  and (g_med is None or g_med["pass"])),
                                     "flux_form": FLUX_FORM_NOTE[flux_form],
                                     "wall_stress_note":
                                         "wall stress error relative to max(FP64 peak, 1e-6 of "
                                         "the solid's shear modulus); the plain relative error "
                                         "is beside it"}
        if (world == 1 and kw.get("model", 0) == 5 and flux_form != 0 and not args.no_fp32_form
                and not args.no_reference_form):
            # the same FP32-flux error report with the reference's own m5 flux
            kref = dict(kw, flux_form=0)
            s64 = Solver(device=local, **kref)
            s64.set_mesh(mesh)
            s64.upload_state(S0)
            dt_ref = dt * REFERENCE_FLUX_CFL / cfg.get("cfl", REFERENCE_FLUX_CFL)
            rf = measure_fp32_form(mesh, S0, dt_ref, kref, args, dev, s64)
            s64.close()
            line["reference_flux_form"] = {k: rf[k] for k in (
                "value", "ms_per_step", "flux_form", "error_vs_fp64", "gate",
                "fp64_sensitivity_floor", "error_growth")}
            line["reference_flux_form"]["cfl"] = REFERENCE_FLUX_CFL
        line["clocks"] = clocks.stop()
        print(json.dumps(line), flush=True)
    else:
        clocks.stop()
    solver.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def measure_amr(mesh, S0, dt, kw, args, dev, amr_cfg, alg_bytes, roofline_of, kernel_times,
                stream64) -> dict:
    """The metric's two forms over the time loop with mesh adaptation, both from the
    criterion-adapted mesh and state: plain FP64 with plain AMR (the reference's loop,
    meshadaptation every `every` steps) and the FP32-flux form with learned AMR (network
    every `infer_every` steps, the criterion as judge every `every` steps, regrids only when it finds
    cells to refine or after three skips).  Returns the keys of the headline line."""
    import torch

    from forestfv_public_gb300 import Solver
    from forestfv_public_gb300.amr import AdaptiveRun
    from forestfv_public_gb300.fields import error_report_meshes
    ind, train = train_wall_indicator(kw, dev, amr_cfg)
    tags = tuple(amr_cfg["tags"])
    every, thr = amr_cfg["every"], amr_cfg["threshold"]
    si_max = tags[13] if tags[11] == 1 else 0
    judge_launches = (si_max + 2) if tags[11] == 1 else 3

    def fresh(precision):
        s = Solver(device=dev.index, precision=precision, **kw)
        s.set_mesh(mesh)
        s.upload_state(S0)
        return s

    # plain FP64 + plain AMR
    sp = fresh(0)
    plain = AdaptiveRun(sp, tags, every=every)
    st_p = torch.cuda.ExternalStream(sp.stream_handle(), device=dev)
    sec_p, cu_p, _, _ = timed_amr_loop(sp, plain, dt, args.steps, args.warmup, st_p)
    # FP32 flux + learned AMR
    sl = fresh(1)
    learned = AdaptiveRun(sl, tags, every=every, indicator=ind, threshold=thr,
                          infer_every=amr_cfg.get("infer_every", 1))
    st_l = torch.cuda.ExternalStream(sl.stream_handle(), device=dev)
    sec_l, cu_l, _, _ = timed_amr_loop(sl, learned, dt, args.steps, args.warmup, st_l)
    mu = kw.get("mu")
    solid = 0 if mu is not None and mu[0] != 0.0 else None
    err = error_report_meshes(sl.mesh, sl.download_state(), sp.mesh, sp.download_state(),
                              kw["gamma"], kw["pinf"], mu, kw["amin"], solid)
    roof32 = roofline_of(kernel_times(sl, 3), sl.mesh.n,
                         "FP32-flux form; its face kernel mixes FP32 arithmetic with the FP64 "
                         "pressure recovery of the critical slots")
    # the learned form end to end: state uploaded from and downloaded to pinned host memory
    # around every step of the same loop
    se = fresh(1)
    e2e_run = AdaptiveRun(se, tags, every=every, indicator=ind, threshold=thr,
                            infer_every=amr_cfg.get("infer_every", 1))
    st_e = torch.cuda.ExternalStream(se.stream_handle(), device=dev)
    sec_e, cu_e, h2d, d2h = timed_amr_loop(se, e2e_run, dt, args.steps, args.warmup, st_e,
                                           host=True)
    value = cu_l / sec_l
    plain_value = cu_p / sec_p
    out = {
        "value": value, "ms_per_step": 1e3 * sec_l / args.steps,
        "dtype": "f32 flux, f64 state and residuals",
        "form": "FP32-flux + learned AMR",
        "e2e": {"value": cu_e / sec_e, "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps, "steps": args.steps},
        "roofline": roof32,
        "gpu_launches": amr_launches(sl, learned.stats, judge_launches),
        "plain_fp64_amr": {"value": plain_value, "unit": UNIT,
                           "ms_per_step": 1e3 * sec_p / args.steps,
                           "amr": plain.stats.as_dict()},
        "learned_amr": {"amr": learned.stats.as_dict(), "indicator_training": train,
                        "every": every, "horizon": amr_cfg["horizon"], "threshold": thr,
                        "infer_every": amr_cfg.get("infer_every", 1),
                        "error_vs_plain_fp64_amr": err,
                        "gate": accuracy_gate(err, args.steps, mu),
                        "speedup_vs_plain_fp64_amr": value / plain_value},
    }
    for s in (sp, sl, se):
        s.close()
    ind.close()
    return out


def run_stress(args) -> None:
    """The stress test (config5, 40.8 M cells): one solver context at a time (a context holds
    ~145 GB of device buffers at this size, so the legs that keep two or three alive do not
    fit): the plain FP64 form, then the FP32-flux form, each timed with CUDA events on its
    stream over `steps` steps after `warmup`, its per-kernel times, and the FP32 form's
    error against the FP64 form after the same steps from host copies of both states."""
    import torch

    from forestfv_public_gb300 import Solver
    from forestfv_public_gb300.fields import error_report
    dev = torch.device("cuda", 0)
    mesh, S0, dt, cfg, kw, alg_bytes, _ = WORKLOADS[args.workload]()
    flux_form = FLUX_FORMS[args.flux_form]
    kw["flux_form"] = flux_form
    cfg["flux_form"] = FLUX_FORM_NOTE[flux_form]
    out = {}
    clocks = ClockSampler()
    clocks.start()
    for name, precision in (("plain_fp64_form", 0), ("fp32_flux_form", 1)):
        s = Solver(device=0, precision=precision, **kw)
        s.set_mesh(mesh)
        s.upload_state(S0)
        stream = torch.cuda.ExternalStream(s.stream_handle(), device=dev)
        s.step(dt, args.warmup)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
        s.step_async(dt, args.steps)
        e1.record(stream)
        s.sync()
        torch.cuda.synchronize(dev)
        t_ms = e0.elapsed_time(e1)
        per = {}
        for _ in range(2):
            for irk in (1, 2):
                for k, v in s.profile_stage(irk, dt).items():
                    per.setdefault(k, []).append(v)
        mean_ms = {k: sum(v) / len(v) for k, v in per.items()}
        dom = max(mean_ms, key=mean_ms.get)
        peak, peak_kind = peak_hbm()
        achieved = alg_bytes.get(dom, 0) * mesh.n / (mean_ms[dom] / 1e3) / 1e9
        out[name] = {"value": mesh.n * args.steps / (t_ms / 1e3), "unit": UNIT,
                     "ms_per_step": t_ms / args.steps, "kernel_mean_ms_per_stage": mean_ms,
                     "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved,
                                  "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                                  "traffic": ncu_summary(dom, mesh.n, "config3")[0],
                                  "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
                     "gpu_launches": s.launches_per_step() * args.steps}
        out[name]["state"] = s.download_state()
        s.close()
    e = error_report(out["fp32_flux_form"].pop("state"), out["plain_fp64_form"].pop("state"),
                     kw["gamma"], kw["pinf"], kw["mu"], kw["amin"], 0)
    out["fp32_flux_form"]["error_vs_fp64"] = e
    out["fp32_flux_form"]["gate"] = accuracy_gate(e, args.steps + args.warmup, kw.get("mu"))
    f32, f64 = out["fp32_flux_form"], out["plain_fp64_form"]
    line = {"metric": METRIC, "value": f32["value"], "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": f32["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 flux, f64 state and residuals", "data": "synthetic", "config": cfg,
            "form": "FP32-flux form (no AMR loop: one solver context at a time at this size)",
            "roofline": f32["roofline"], "gpu_launches": f32["gpu_launches"],
            "speedup_vs_plain_fp64": f32["value"] / f64["value"],
            "plain_fp64_form": f64, "fp32_flux_form": f32, "clocks": clocks.stop()}
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--workload", default="config3", choices=tuple(WORKLOADS))
    ap.add_argument("--cpu-rounds", type=int, default=3,
                    help="rounds of the CPU baseline (all host cores, one range each); 0 skips it")
    ap.add_argument("--flux-form", default="consistent", choices=tuple(FLUX_FORMS),
                    help="model 5's flux: the reference's as written, or made consistent "
                         "(include/ffv.h FFV_FLUX_CONSISTENT); the default is the one whose "
                         "FP32-flux form meets the metric's accuracy condition")
    ap.add_argument("--loops", action="store_true",
                    help="config5: the full set of legs (AMR loops, error-growth solvers side by "
                         "side) instead of the one-context-at-a-time stress leg")
    ap.add_argument("--no-reference-form", action="store_true",
                    help="skip the FP32-flux error report with the reference's own flux")
    ap.add_argument("--no-amr", action="store_true",
                    help="skip the time loops with mesh adaptation (headline = plain FP64)")
    ap.add_argument("--no-fp32-form", action="store_true",
                    help="skip the FP32-flux form's throughput and error report")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload.startswith("config5") and not args.loops:
        run_stress(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
