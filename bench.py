#!/usr/bin/env python3
"""Throughput benchmark of the explicit FV step (cell-updates per second).

Default workload (--workload config2): the plain FP64 form on the two-phase gas-bubble
collapse in liquid -- liquid stiffened gas (gamma 4.4, p_inf 6e8, rho 1000, p 5e6), gas
sphere (gamma 1.4, rho 1, p 1e5) of radius 0.1 with a tanh interface over two finest cells
and seeded radius harmonics l <= 8 (relative amplitude 1e-3), 2^3 trees refined from level
5 to level 8 around the interface (2.30 M cells, 2:1 balanced), transmissive sides, model
5 (six-equation, 2 materials, NEQ 18), MUSCL-HLLC with face-state relaxation, PRELAX 3,
RK_STEPS 2, FP64.  dt is CFL 0.01 on the liquid sound speed at the finest cell: the
reference's model-5 scheme stops with NaN wave speeds on this problem at larger steps (its
own C code, reproduced bit for bit by the oracle); work per step does not depend on dt.
`--workload config1` is the 32^3 Sod problem of model 0.

One benchmark step is one time step (all RK stages) over the whole mesh; one cell-update
is one cell advanced one time step.

  value      graph-launched steps, state resident in HBM, CUDA events on the solver's
             stream around every step; config2's state (331 MB) exceeds L2, config1's is
             flushed from L2 (256 MiB write) between steps
  e2e        the same through the public API with host buffers: every step uploads the
             state from pinned host memory, runs the step and downloads the state
  roofline   the dominant kernel's algorithmic bytes per launch over its mean duration,
             per-kernel CUDA events on the solver's stream (ffv_profile_stage)
  cpu_baseline  the oracle's C restatement of the reference algorithm, one core, on a
             bounded sample (same physics, smaller mesh)

`--impl reference` times the reference algorithm on the host cores instead (the C
restatement in oracle/, one process per core, each on the same bounded sample).
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


def wl_config2(small: bool = False, medium: bool = False):
    from forestfv_public_gb300 import workloads as W
    if small:  # CPU sample: same physics, levels 4..6
        mesh, S0, p = W.bubble_config2(lmin=4, lmax=6, band_cells=2.0)
        hmin = 0.5 / (1 << 5)
    elif medium:  # profiler captures: levels 4..7, 0.36 M cells
        mesh, S0, p = W.bubble_config2(lmin=4, lmax=7, band_cells=12.0)
        hmin = 0.5 / (1 << 6)
    else:
        mesh, S0, p = W.bubble_config2()
        hmin = 0.5 / (1 << 7)
    dt = 0.01 * hmin / C_LIQUID
    neq = S0.shape[0]
    cfg = {"workload": "config2 bubble collapse in liquid, model 5 (2 materials), levels 5-8 AMR, "
                       "plain FP64, MUSCL-HLLC, PRELAX 3, RK2",
           "cells": int(mesh.n), "levels": sorted(int(x) for x in np.unique(mesh.level)),
           "neq": neq, "dt": float(dt), "cfl": 0.01, "parallelism": "single GPU",
           "l2": "state 331 MB > L2 (129 MB): no flush needed"}
    # algorithmic bytes per cell of each kernel (compulsory traffic, neighbour re-reads excluded)
    d = 8 * neq
    alg = {"m5_recon_face": d + 28 + 6 * d,
           "m5_face_flux": 6 * d + d + 28 + 6 * d + 6 * 3 * 8 + 6 * 8,
           "m5_cell_update": d + 6 * d + 6 * 3 * 8 + d + 28 + d + d + 1,
           "m5_relax_cell": d + d + 1}
    return mesh, S0, dt, cfg, _bubble_solver_kwargs(p), alg, False


def wl_config1(small: bool = False):
    from forestfv_public_gb300 import Mesh, uniform_leaves
    trees, level = (4, 4, 4), 4
    mesh = Mesh(trees, uniform_leaves(trees, level))
    S0 = sod_state(mesh.centroids())
    dt = 0.4 * (1.0 / 32.0) / np.sqrt(1.4)
    cfg = {"workload": "config1 Sod 32^3, model 0, plain FP64, MUSCL-HLLC, RK2, CFL 0.4",
           "cells": int(mesh.n), "trees": list(trees), "level": level, "dt": float(dt),
           "parallelism": "single GPU",
           "l2": "flushed between timed steps (256 MiB write); state 1.3 MB < L2"}
    alg = {"m0_recon": 40 + 28 + 240, "m0_flux_rk<2>": 240 + 40 + 40 + 28 + 40}
    return mesh, S0, float(dt), cfg, dict(model=0), alg, True


def wl_config2m(small: bool = False):
    """config2 physics on a 0.36 M-cell mesh (levels 4-7): the size profiler captures use."""
    out = wl_config2(small=small, medium=not small)
    out[3]["workload"] = out[3]["workload"].replace("levels 5-8", "levels 4-7 (medium size)")
    return out


WORKLOADS = {"config2": wl_config2, "config1": wl_config1, "config2m": wl_config2m}


# ------------------------------------------------------------------------------ helpers
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


def ncu_summary(kernel: str, cells: int):
    """(DRAM bytes per launch, FP64-pipe % busy) of a kernel from the committed ncu summary
    (bytes per cell x cells); None where the kernel has no capture."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for ln in open(p):
            t = ln.split()
            if len(t) >= 2 and not ln.startswith("#") and t[0] == kernel:
                return float(t[1]) * cells, (float(t[2]) if len(t) > 2 else None)
    except OSError:
        pass
    return None, None


_CPU_CACHE = {}


def cpu_sample(workload: str, seconds: float = 10.0):
    """Time the oracle's C restatement on the workload's CPU sample, one core."""
    from oracle import pyoracle
    if workload not in _CPU_CACHE:
        mesh, S0, dt, _, kw, _, _ = WORKLOADS[workload](small=True)
        _CPU_CACHE[workload] = (mesh, S0, dt, kw, pyoracle.OracleMesh(mesh.export()))
    mesh, S0, dt, kw, om = _CPU_CACHE[workload]
    S = np.ascontiguousarray(S0.T)

    def adv(S, k):
        if kw.get("model", 0) == 5:
            m5 = dict(avf_lim=kw["avf_lim"], prelax=kw["prelax"], amin=kw["amin"],
                      pinf=list(kw["pinf"]), gamma=list(kw["gamma"]), mu=list(kw["mu"]))
            return pyoracle.m5_advance(om, S, dt, k, m5)
        return pyoracle.m0_advance(om, S, dt, k)

    t0 = time.perf_counter()
    S = adv(S, 1)
    one = time.perf_counter() - t0
    steps = max(1, min(200, int(seconds / max(one, 1e-6))))
    t0 = time.perf_counter()
    adv(S, steps)
    el = time.perf_counter() - t0
    return mesh.n * steps / el, steps, mesh.n


def _cpu_worker(args):
    workload, seconds = args
    return cpu_sample(workload, seconds)


# ------------------------------------------------------------------------------ arms
def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from multiprocessing import get_context
    from oracle import pyoracle
    pyoracle.lib()  # build once before the workers start
    cores = os.cpu_count() or 1
    full_cfg = WORKLOADS[args.workload]()[3]
    per_step = []
    ctx = get_context("spawn")
    per_step_s = max(0.5, min(3.0, 120.0 / max(1, args.steps)))
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_cpu_worker, [(args.workload, 0.2)] * cores)
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, [(args.workload, per_step_s)] * cores)
            el = time.perf_counter() - t0
            per_step.append(sum(r[1] * r[2] for r in res) / el)
    value = statistics.median(per_step)
    steps, n = res[0][1], res[0][2]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "dtype": "f64", "data": "synthetic", "config": full_cfg, "vs_baseline": None,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} processes x {steps} steps of a {n}-cell mesh of the "
                                   "same problem (oracle C restatement of the reference "
                                   "algorithm; the reference's own binary is not built on "
                                   "this host)"},
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

    def advance(solver, S):
        solver.upload_state(S)
        solver.step(dt, args.steps)
        return solver.download_state()

    mu = kw.get("mu")
    solid = 0 if mu is not None and mu[0] != 0.0 else None
    ref = advance(fp64_solver, S0)
    err = error_report(advance(s32, S0), ref, kw["gamma"], kw["pinf"], mu, kw["amin"], solid)
    rng = np.random.default_rng(20261203)
    Sp = S0 * (1.0 + FP32_PERTURBATION * rng.uniform(-1.0, 1.0, S0.shape))
    floor = error_report(advance(fp64_solver, Sp), ref, kw["gamma"], kw["pinf"], mu, kw["amin"],
                         solid)
    s32.close()
    return {"value": mesh.n * args.steps / (t_ms / 1e3), "unit": UNIT,
            "ms_per_step": t_ms / args.steps, "kernel_mean_ms_per_stage": mean_ms,
            "error_vs_fp64": err, "error_steps": args.steps,
            "fp64_sensitivity_floor": {"perturbation": FP32_PERTURBATION, **floor},
            "note": "error of the FP32-flux form against the FP64 form after error_steps steps, "
                    "beside the FP64 form's own change when its initial state is perturbed by "
                    "1e-7 relative: the reference's model-5 scheme amplifies rounding-level "
                    "differences, so the FP32 form is judged against that floor"}


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
    solver = Solver(device=local, **kw)
    solver.set_mesh(mesh)
    solver.upload_state(S0)
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
    clock_info = clocks.stop()
    t_ms = sum(a.elapsed_time(b) for a, b in ev)
    if world > 1:
        t = torch.tensor([t_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_ms = float(t.item())
    value = world * mesh.n * args.steps / (t_ms / 1e3)

    # per-kernel durations for the roofline (same stages, events around every kernel)
    per_kernel = {}
    nprof = max(3, min(args.steps, 10))
    for _ in range(nprof):
        for irk in (1, 2):
            if flush is not None:
                with torch.cuda.stream(stream):
                    flush.zero_()
            for name, ms in solver.profile_stage(irk, dt).items():
                per_kernel.setdefault(name, []).append(ms)
    mean_ms = {k: sum(v) / len(v) for k, v in per_kernel.items()}
    dom = max(mean_ms, key=mean_ms.get)
    peak, peak_kind = peak_hbm()
    alg = alg_bytes.get(dom, 0) * mesh.n
    achieved = alg / (mean_ms[dom] / 1e3) / 1e9
    step_ms = sum(mean_ms.values())
    traffic, fp64_pct = ncu_summary(dom, mesh.n)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "kernel": dom,
                "fp64_pipe_busy_pct_ncu": fp64_pct,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst)",
                "kernel_mean_ms_per_stage": mean_ms,
                "kernel_share": {k: v / step_ms for k, v in mean_ms.items()},
                "alg_bytes_per_launch": alg,
                "note": "the FP64 kernels are FP64-pipe bound (GB300 FP64 = 1/64 FP32), "
                        "see profiles/"}

    # end to end through the public API with pinned host buffers
    host = torch.empty((neq, mesh.n), dtype=torch.float64, pin_memory=True).numpy()
    host[:] = S0
    torch.cuda.synchronize(dev)
    e2e_steps = max(1, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.upload_state(host)
        solver.step(dt, 1)
        host[:] = solver.download_state()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * mesh.n * e2e_steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": neq * 8 * mesh.n, "d2h_bytes_per_step": neq * 8 * mesh.n,
           "steps": e2e_steps}

    if rank == 0:
        cpu = None
        if world == 1:
            rate, csteps, n = cpu_sample(args.workload, args.cpu_seconds)
            cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"{csteps} steps of a {n}-cell mesh of the same problem, oracle C "
                             "restatement of the reference algorithm"}
        fp32 = None
        if world == 1 and kw.get("model", 0) == 5 and not args.no_fp32_form:
            fp32 = measure_fp32_form(mesh, S0, dt, kw, args, dev, solver)
            fp32["speedup_vs_fp64"] = fp32["value"] / value
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clock_info,
            "gpu_launches": solver.launches_per_step() * args.steps,
        }
        if fp32 is not None:
            line["fp32_flux_form"] = fp32
        print(json.dumps(line), flush=True)
    solver.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--workload", default="config2", choices=tuple(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-fp32-form", action="store_true",
                    help="skip the FP32-flux form's throughput and error report")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
