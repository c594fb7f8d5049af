"""Throughput of the JustPIC particle-in-cell hot path on one GB300.

Workload (default): 2D temperature advection, FP64, 1024 x 1024 cells, 24
particles per cell (max 48, min 12, seeded uniform placement), rigid-body
rotation velocity on the staggered ghost-node grids, vertex temperature
exp(-((x-0.5)^2+(y-0.75)^2)/0.01) carried by the particles. One step is the
reference miniapp cycle (test/test_2D.jl:516-524): particle2grid!,
advection! (RK2), move_particles!, inject_particles!, grid2particle!.

Metric: particle-steps/s = live particles x steps / device time. ``value`` is
measured with the particle data resident in HBM and asynchronous calls;
``e2e`` goes through the public API in its default synchronous mode with the
velocity grids copied from pinned host memory each step and the gridded
temperature read back each step.

``--impl reference`` times the reference's CPU algorithm (the FP64 C
restatement in oracle/, all host threads; Julia is not available) on the same
workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD = "C2"
METRIC = "particle-steps/s on 1 GB300, FP32-offset vs FP64 at stated error; HBM % of peak"
UNIT = "particle-steps/s"

# Algorithmic bytes per live particle of each call (2D FP64, one particle field):
# every live particle's data once per call, the Bool index at 1 byte per slot
# (2 bytes per live particle at 24 of 48 slots), grid arrays once per call
# amortised over the particles; movers (fraction m) re-read and re-write their
# coordinates and field.
BYTES = {
    "advection!": lambda m: 16 + 16 + 2 + 0.7,
    "move_particles!": lambda m: 16 + 2 + m * (2 * (16 + 8) + 2),
    "inject_particles!": lambda m: 16 + 2,
    "grid2particle!": lambda m: 16 + 2 + 8 + 0.35,
    "particle2grid!": lambda m: 16 + 2 + 8 + 0.35,
}
LAUNCHES_PER_STEP = {"particle2grid!": 1, "advection!": 1, "move_particles!": 11, "inject_particles!": 5,
                     "grid2particle!": 1}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._thread = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._thread.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, name in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def movers_fraction(jp, p, torch):
    """Fraction of live particles outside their cell (after an advection!)."""
    idx = p.index.data.bool()
    m, live = 0, int(idx.sum())
    ncells = p.index.data.shape[1]
    cells = torch.arange(ncells, device="cuda")
    out = torch.zeros_like(idx)
    stride = 1
    for d in range(p.ndim):
        n = p.ni[d]
        I = (cells // stride) % n
        stride *= n
        xv = torch.as_tensor(np.asarray(p.xvi[d]), device="cuda")
        lo, hi = xv[I], xv[I + 1]
        x = p.coords[d].data
        out |= ~((x > lo) & (x < hi))
    m = int((out & idx).sum())
    return m / max(1, live)


def run_ours(args):
    import torch

    import justpic_gb300 as jp
    from justpic_gb300 import workloads as W

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    jp._native.load()

    cfg = W.setup(WORKLOAD, args.ni and (args.ni, args.ni))
    g = cfg["grid"]
    Vx, Vy = cfg["V"]
    dt = cfg["dt"]
    p = jp.init_particles(jp.CUDABackend, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], *g["grid_v"],
                          seed=jp.DEFAULT_SEED + rank)
    pT, = jp.init_cell_arrays(p, 1)
    V = (jp.TA("CUDA")(Vx), jp.TA("CUDA")(Vy))
    T = jp.TA("CUDA")(cfg["T"])
    method = jp.RungeKutta2()
    jp.grid2particle_(pT, T, p)

    stream = torch.cuda.current_stream()
    ops = ["particle2grid!", "advection!", "move_particles!", "inject_particles!", "grid2particle!"]

    def step(ev=None):
        calls = [
            lambda: jp.particle2grid_(T, pT, p),
            lambda: jp.advection_(p, method, V, dt),
            lambda: jp.move_particles_(p, (pT,)),
            lambda: jp.inject_particles_(p, (pT,)),
            lambda: jp.grid2particle_(pT, T, p),
        ]
        for k, call in enumerate(calls):
            if ev is not None:
                ev[k][0].record(stream)
            call()
            if ev is not None:
                ev[k][1].record(stream)

    # movers fraction of this workload (measured once, outside the timed region)
    jp.particle2grid_(T, pT, p)
    jp.advection_(p, method, V, dt)
    m = movers_fraction(jp, p, torch)
    jp.move_particles_(p, (pT,))
    jp.inject_particles_(p, (pT,))
    jp.grid2particle_(pT, T, p)

    # ---- device-resident throughput (asynchronous calls) ----
    jp.set_synchronous(p, False)
    for _ in range(args.warmup):
        step()
    jp.synchronize(p)
    live0 = int(p.index.data.sum())
    events = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)] for _ in ops]
              for _ in range(args.steps)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0.record(stream)
        for k in range(args.steps):
            step(events[k])
        t1.record(stream)
        torch.cuda.synchronize()
    jp.synchronize(p)
    if world > 1:
        torch.distributed.barrier()
    live1 = int(p.index.data.sum())
    elapsed = t0.elapsed_time(t1) / 1e3
    if world > 1:
        tt = torch.tensor([elapsed], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        elapsed = float(tt)
    live = 0.5 * (live0 + live1)
    value = live * args.steps * world / elapsed
    op_ms = {op: float(np.mean([events[k][i][0].elapsed_time(events[k][i][1]) for k in range(args.steps)]))
             for i, op in enumerate(ops)}

    # ---- end to end through the public API (synchronous, host buffers) ----
    jp.set_synchronous(p, True)
    hVx = torch.from_numpy(np.ascontiguousarray(Vx.T)).pin_memory()
    hVy = torch.from_numpy(np.ascontiguousarray(Vy.T)).pin_memory()
    hT = torch.empty(tuple(reversed(T.shape)), dtype=torch.float64).pin_memory()
    dVx = torch.empty_like(hVx, device="cuda")
    dVy = torch.empty_like(hVy, device="cuda")
    e2e_steps = max(1, min(args.steps, 50))
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for _ in range(e2e_steps):
        dVx.copy_(hVx, non_blocking=True)
        dVy.copy_(hVy, non_blocking=True)
        Vstep = (dVx.T, dVy.T)
        jp.particle2grid_(T, pT, p)
        jp.advection_(p, method, Vstep, dt)
        jp.move_particles_(p, (pT,))
        jp.inject_particles_(p, (pT,))
        jp.grid2particle_(pT, T, p)
        hT.copy_(T.T, non_blocking=False)
    torch.cuda.synchronize()
    e2e_time = time.perf_counter() - w0
    e2e_value = live * e2e_steps * world / e2e_time

    # ---- roofline of the dominant call ----
    peak, peak_kind = _peaks()
    dom = max(op_ms, key=op_ms.get)
    bytes_dom = BYTES[dom](m) * live
    achieved = bytes_dom / (op_ms[dom] / 1e3) / 1e9
    step_bytes = sum(BYTES[o](m) for o in ops) * live
    step_gbs = step_bytes / (elapsed / args.steps) / 1e9

    result = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded analytic rigid-rotation workload; no public dataset exists)",
        "config": {
            "workload": "C2: 2D temperature advection FP64, 1024x1024 cells, 24/48/12 particles per cell, "
                        "rigid rotation, RK2, step = particle2grid!+advection!+move_particles!+"
                        "inject_particles!+grid2particle!",
            "cells": [1024, 1024],
            "live_particles": live,
            "dt": dt,
            "movers_fraction": m,
            "l2": "inputs larger than L2 (coordinates alone 805 MB)",
            "parallelism": "replicas" if world > 1 else "single GPU",
        },
        "per_call_ms": op_ms,
        "step_algorithmic_gbs": step_gbs,
        "roofline": {
            "bound": "hbm",
            "kernel": dom,
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
            else "fallback 6.8 TB/s",
            "bytes_per_particle": BYTES[dom](m),
            "traffic": None,
        },
        "e2e": {
            "value": e2e_value,
            "unit": UNIT,
            "h2d_bytes_per_step": int(hVx.numel() * 8 + hVy.numel() * 8),
            "d2h_bytes_per_step": int(hT.numel() * 8),
            "steps": e2e_steps,
            "mode": "public API, synchronous calls, velocity in / vertex temperature out each step",
        },
        "gpu_launches": sum(LAUNCHES_PER_STEP.values()) * args.steps,
        "clocks": clocks.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(result))


def _cpu_setup():
    from justpic_gb300 import workloads as W
    from oracle import oracle as O

    cfg = W.setup(WORKLOAD)
    g = cfg["grid"]
    grids = tuple(tuple(np.asarray(x) for x in comp) for comp in g["grid_v"])
    o = O.OracleParticles(grids, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], uniform=True)
    o.init_particles()
    oT = o.cell_array()
    T = np.asfortranarray(cfg["T"].copy())
    o.grid2particle(oT, T)
    V = cfg["V"]
    dt = cfg["dt"]

    def step():
        o.particle2grid(T, oT)
        o.advection(O.RK2, 0.5, V, dt)
        o.move_particles((oT,))
        o.inject_particles((oT,))
        o.grid2particle(oT, T)

    return o, step


def cpu_baseline(seconds=20.0, max_steps=None):
    """The FP64 C restatement of the reference's CPU path, all host threads, on
    the same workload; times whole steps until ``seconds`` of CPU work."""
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    O.set_threads(cores)
    o, step = _cpu_setup()
    step()  # warm-up (page faults, thread pool)
    n, t = 0, 0.0
    while t < seconds and (max_steps is None or n < max_steps):
        live = int(o.index.sum())
        w0 = time.perf_counter()
        step()
        t += time.perf_counter() - w0
        n += 1
    value = live * n / t
    return {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} full C2 steps (1024x1024 cells, ~25M particles) in {t:.1f} s with {cores} OpenMP "
                      "threads; C restatement of the reference's FP64 CPU path (Julia is not available)"}


def run_reference(args):
    world, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    O.set_threads(cores)
    o, step = _cpu_setup()
    for _ in range(max(0, min(args.warmup, 1))):
        step()
    budget = 90.0
    n, t = 0, 0.0
    live_sum = 0
    while n < args.steps and (t < budget or n == 0):
        live_sum += int(o.index.sum())
        w0 = time.perf_counter()
        step()
        t += time.perf_counter() - w0
        n += 1
    value = live_sum / t
    print(json.dumps({
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": n,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t / n,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded analytic rigid-rotation workload)",
        "config": {"workload": "C2: 2D temperature advection FP64, 1024x1024 cells, 24/48/12 particles per "
                               "cell, rigid rotation, RK2, five calls per step", "cells": [1024, 1024]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{n} of {args.steps} requested full steps timed (capped at {budget:.0f} s); "
                                   "FP64 C restatement of JustPIC.CPU (Julia is not installed)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ni", type=int, default=None,
                    help="cells per axis instead of 1024 (small cases for ncu captures; not a bench line)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
