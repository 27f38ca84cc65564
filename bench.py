#!/usr/bin/env python3
"""Throughput benchmark of the explicit FV step (cell-updates per second).

Workload: the plain-method Sod problem of a 32^3 uniform forest (4^3 trees at level 4),
ideal gas, transmissive sides, MUSCL-HLLC, RK_STEPS 2, FP64, fixed dt = CFL 0.4 on the
initial state.  One benchmark step is one time step (both RK stages) over the whole
mesh; one cell-update is one cell advanced one time step.

  value      graph-launched steps, state resident in HBM, CUDA events on the solver's
             stream around every step, L2 flushed (256 MiB write) between steps
  e2e        the same through the public API with host buffers: every step uploads the
             state from pinned host memory, runs the step and downloads the state
  roofline   the dominant kernel's algorithmic bytes per launch over its mean duration,
             per-kernel CUDA events on the solver's stream (ffv_profile_stage)
  cpu_baseline  the oracle's C restatement of the reference algorithm, one core, on a
             bounded number of steps of the same mesh

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
NEQ = 5
L2_FLUSH_BYTES = 256 << 20


def sod_state(cent: np.ndarray, gamma: float = 1.4) -> np.ndarray:
    """Sod initial state in SoA, as the reference's m0_init_S (init_S.c:3-16) forms it."""
    left = cent[:, 0] < 0.5
    S = np.empty((NEQ, len(cent)))
    for mask, (rho, u, v, w, p) in ((left, SOD[0]), (~left, SOD[1])):
        e_int = (p + gamma * 0.0) / (rho * (gamma - 1.0))
        S[0, mask] = rho
        S[1, mask] = rho * u
        S[2, mask] = rho * v
        S[3, mask] = rho * w
        S[4, mask] = rho * (e_int + 0.5 * (u * u + v * v + w * w))
    return S


def workload():
    from forestfv_public_gb300 import Mesh, uniform_leaves
    trees, level = (4, 4, 4), 4
    mesh = Mesh(trees, uniform_leaves(trees, level))
    S0 = sod_state(mesh.centroids())
    dt = 0.4 * (1.0 / 32.0) / np.sqrt(1.4)
    cfg = {"workload": "sod32-uniform-fp64 (config 1: 32^3 Sod, MUSCL-HLLC, RK2, CFL 0.4)",
           "cells": int(mesh.n), "trees": list(trees), "level": level, "rk_steps": 2,
           "order": 2, "dt": float(dt), "parallelism": "single GPU",
           "l2": "flushed between timed steps (256 MiB write); state 1.3 MB < L2"}
    return mesh, S0, float(dt), cfg


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


def ncu_traffic(kernel: str, cells: int):
    """DRAM bytes per launch from the committed ncu summary (bytes per cell x cells)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for ln in open(p):
            t = ln.split()
            if len(t) >= 2 and not ln.startswith("#") and t[0] == kernel:
                return float(t[1]) * cells
    except OSError:
        pass
    return None


# algorithmic bytes per cell of each kernel (compulsory traffic; neighbour re-reads excluded)
ALG_BYTES = {
    # S (5 doubles) + info word + 6 neighbour slots in, 6 face states x 5 doubles out
    "m0_recon": 8 * NEQ + 4 + 24 + 6 * NEQ * 8,
    # own 6 face states + S + SN + info + neighbour slots in, S out (SN out in stage 1)
    "m0_flux_rk<2>": 6 * NEQ * 8 + 8 * NEQ + 8 * NEQ + 4 + 24 + 8 * NEQ,
}


_CPU_CACHE = {}


def cpu_sample(seconds: float = 10.0):
    """Time the oracle's C restatement on the bench mesh, one core, ~`seconds` of work."""
    from oracle import pyoracle
    if "mesh" not in _CPU_CACHE:
        mesh, S0, dt, _ = workload()
        _CPU_CACHE.update(mesh=mesh, S0=S0, dt=dt, om=pyoracle.OracleMesh(mesh.export()))
    mesh, S0, dt, om = (_CPU_CACHE[k] for k in ("mesh", "S0", "dt", "om"))
    S = np.ascontiguousarray(S0.T)
    t0 = time.perf_counter()
    S = pyoracle.m0_advance(om, S, dt, 1)
    one = time.perf_counter() - t0
    steps = max(1, min(200, int(seconds / max(one, 1e-6))))
    t0 = time.perf_counter()
    pyoracle.m0_advance(om, S, dt, steps)
    el = time.perf_counter() - t0
    return mesh.n * steps / el, steps, mesh.n


def _cpu_worker(args):
    seconds, = args
    return cpu_sample(seconds)


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from multiprocessing import get_context
    from oracle import pyoracle
    pyoracle.lib()  # build once before forking workers
    cores = os.cpu_count() or 1
    _, _, _, cfg = workload()
    per_step = []
    ctx = get_context("spawn")
    per_step_s = max(0.2, min(3.0, 120.0 / max(1, args.steps)))
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_cpu_worker, [(0.2,)] * cores)
        for _ in range(args.steps):
            t0 = time.perf_counter()
            res = pool.map(_cpu_worker, [(per_step_s,)] * cores)
            el = time.perf_counter() - t0
            per_step.append(sum(r[1] * r[2] for r in res) / el)
    value = statistics.median(per_step)
    steps, n = res[0][1], res[0][2]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "dtype": "f64", "data": "synthetic", "config": cfg, "vs_baseline": None,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} processes x {steps} steps of the {n}-cell mesh "
                                   "(oracle C restatement of the reference algorithm; the "
                                   "reference's own binary cannot be built on this host)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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

    mesh, S0, dt, cfg = workload()
    solver = Solver(device=local)
    solver.set_mesh(mesh)
    solver.upload_state(S0)
    stream = torch.cuda.ExternalStream(solver.stream_handle(), device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    # warm-up (also builds the step graph)
    solver.step(dt, args.warmup)

    # ---- device throughput: one event pair per step, L2 flushed between steps ----
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = ClockSampler()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[k][0].record(stream)
        solver.step_async(dt, 1)
        ev[k][1].record(stream)
    solver.sync()
    torch.cuda.synchronize(dev)
    clock_info = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    t_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([t_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_ms = float(t.item())
    value = world * mesh.n * args.steps / (t_ms / 1e3)

    # ---- per-kernel durations for the roofline (same stages, events per kernel) ----
    per_kernel = {}
    for _ in range(max(3, args.steps)):
        for irk in (1, 2):
            with torch.cuda.stream(stream):
                flush.zero_()
            for name, ms in solver.profile_stage(irk, dt).items():
                per_kernel.setdefault(name, []).append(ms)
    mean_ms = {k: sum(v) / len(v) for k, v in per_kernel.items()}
    dom = max(mean_ms, key=mean_ms.get)
    peak, peak_kind = peak_hbm()
    alg = ALG_BYTES.get(dom, 0) * mesh.n
    achieved = alg / (mean_ms[dom] / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": ncu_traffic(dom, mesh.n), "kernel": dom,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst)",
                "kernel_mean_ms": mean_ms, "alg_bytes_per_launch": alg}

    # ---- end to end through the public API with pinned host buffers ----
    host = torch.empty((NEQ, mesh.n), dtype=torch.float64, pin_memory=True).numpy()
    host[:] = solver.download_state()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        solver.upload_state(host)
        solver.step(dt, 1)
        host[:] = solver.download_state()
    e2e_s = time.perf_counter() - t0
    e2e = {"value": world * mesh.n * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": NEQ * 8 * mesh.n, "d2h_bytes_per_step": NEQ * 8 * mesh.n}

    if rank == 0:
        cpu = None
        if world == 1:
            rate, csteps, n = cpu_sample(args.cpu_seconds)
            cpu = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"{csteps} steps of the {n}-cell mesh, oracle C restatement"}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": cfg, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clock_info,
            "gpu_launches": solver.launches_per_step() * args.steps,
        }
        print(json.dumps(line), flush=True)
    solver.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
