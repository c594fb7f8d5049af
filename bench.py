"""Throughput of the JustPIC particle-in-cell hot path on one GB300.

Default workload (C2): 2D temperature advection, FP64, 1024 x 1024 cells, 24
particles per cell (max 48, min 12, seeded uniform placement), rigid-body
rotation velocity on the staggered ghost-node grids, vertex temperature
exp(-((x-0.5)^2+(y-0.75)^2)/0.01) carried by the particles. One step is the
reference miniapp cycle (test/test_2D.jl:516-524): particle2grid!,
advection! (RK2), move_particles!, inject_particles!, grid2particle!.
``--workload C1`` (256^2, stream function, advection! + move_particles!, no
fields) and ``--workload C3`` (128^3, cellular flow + drift, particle2grid!,
advection!, move_particles!, inject_particles!) use the same harness.

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

METRIC = "particle-steps/s on 1 GB300, FP32-offset vs FP64 at stated error; HBM % of peak"
UNIT = "particle-steps/s"

STEPS = {
    "C1": ["advection!", "move_particles!"],
    "C2": ["particle2grid!", "advection!", "move_particles!", "inject_particles!", "grid2particle!"],
    "C3": ["particle2grid!", "advection!", "move_particles!", "inject_particles!"],
    "C4": ["particle2grid!", "advection!", "move_particles!", "inject_particles!", "grid2particle!"],
    "C5": ["advection!", "move_particles!", "inject_particles!"],
}
DESC = {
    "C1": "C1: 2D RK2 advection FP64, 256x256 cells, 24/48/12 particles per cell, stream-function velocity, "
          "step = advection!+move_particles!",
    "C2": "C2: 2D temperature advection FP64, 1024x1024 cells, 24/48/12 particles per cell, rigid rotation, RK2, "
          "step = particle2grid!+advection!+move_particles!+inject_particles!+grid2particle!",
    "C3": "C3: 3D temperature advection FP64, 128^3 cells, 24/48/12 particles per cell, cellular flow + 0.1 z "
          "drift, RK2, step = particle2grid!+advection!+move_particles!+inject_particles!",
    "C4": "C4: 2D, 2048x2048 cells, 24/48/12 particles per cell, stream-function velocity, RK4, "
          "step = particle2grid!+advection!+move_particles!+inject_particles!+grid2particle!",
    "C5": "C5: 2D adjoint, FP64, 512x512 cells, 16/32/8 particles per cell, stream-function velocity plus "
          "N(0, 25^2) node noise, RK2, 100 steps, loss 0.5||particle2grid(T) - T_target||^2, checkpoints every "
          "10 steps, gradients w.r.t. Vx, Vy, T0",
}


def algorithmic_bytes(op, N, nf, m, slots_per_live, grid_bytes_per_live, field_bytes_per_live, vb=8):
    """Bytes per live particle of one call: every live particle's data once,
    the Bool index at 1 byte per slot, grid arrays once per call amortised
    over the particles; movers (fraction m) re-read and re-write their
    coordinates and fields."""
    coords = vb * N
    idx = slots_per_live
    if op == "advection!":
        return 2 * coords + idx + grid_bytes_per_live
    if op == "move_particles!":
        return coords + idx + m * (2 * (coords + vb * nf) + 2)
    if op == "inject_particles!":
        return coords + idx
    if op == "grid2particle!":
        return coords + idx + vb + field_bytes_per_live
    if op == "particle2grid!":
        return coords + idx + vb + field_bytes_per_live
    raise KeyError(op)


# DRAM bytes per live particle of each call: dram__bytes_read.sum +
# dram__bytes_write.sum of the call's kernels (move: classify + colour passes +
# apply; injection: flag + colour passes), averaged over the calls of one ncu
# launch-list capture of the workload at its own size (one pass; ncu flushes L2
# before each launch) and divided by its live particles. The bench multiplies
# by the live particles of its own run; C4 (2048^2, the same calls as C2) takes
# the C2 figures, a resized workload (--ni) its own workload's.
DRAM_BYTES_PER_PARTICLE = {
    ("C1", "f64"): {"advection!": 31.9, "move_particles!": 90.6},
    ("C1", "f32"): {"advection!": 17.4, "move_particles!": 54.8},
    ("C2", "f64"): {"particle2grid!": 99.3, "advection!": 56.9, "grid2particle!": 54.0, "move_particles!": 216.1,
                    "inject_particles!": 60.5},
    ("C2", "f32"): {"particle2grid!": 28.4, "advection!": 29.4, "grid2particle!": 29.2, "move_particles!": 139.0,
                    "inject_particles!": 38.7},
    ("C3", "f64"): {"particle2grid!": 254.7, "advection!": 76.3, "move_particles!": 219.0,
                    "inject_particles!": 188.7},
    ("C3", "f32"): {"particle2grid!": 37.2, "advection!": 40.8, "move_particles!": 142.0,
                    "inject_particles!": 129.9},
}


def fp64_instructions(op, N, method):
    """FP64 instructions per live particle of the interpolating calls, counted
    from their kernels (every FP64 add, multiply and FMA; the bisection and
    range tests run on integer keys, particle2grid!'s weights on the integer
    pipe): advection samples 2 (Euler 1, RK4 4) velocities of N components,
    each N normalisations (subtract, multiply) and 2^N - 1 lerps (2 FMA),
    plus the stage updates; grid2particle! one N-linear sample;
    particle2grid! 2^(N-1) column visits per particle, each forming the
    column's shared squared terms once for its two vertices, then per vertex
    one add and one FMA. None for the integer/memory calls."""
    sample = N * (2 * N + 2 * ((1 << N) - 1))
    if op == "advection!":
        if method == "RungeKutta4":
            return 4 * sample + N * (3 + 3 + 2) + N * 7
        if method == "Euler":
            return sample + 2 * N
        return 2 * sample + 4 * N
    if op == "grid2particle!":
        return 2 * N + 2 * ((1 << N) - 1)
    if op == "particle2grid!":
        per_visit = (2 + 2 + 2 + 2) if N == 2 else (2 + 2 + 1 + 2 + 2 + 2)
        return (1 << (N - 1)) * (per_visit + 2 * 2)
    return None


def launches(op, N):
    return {"advection!": 1, "move_particles!": 2 + 3 ** N, "inject_particles!": 1 + 2 ** N,
            "grid2particle!": 1, "particle2grid!": 1}[op]


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


def _init_ranks(local, backend="nccl"):
    """One process per GPU (torchrun sets RANK/WORLD_SIZE/MASTER_*). The ranks
    are independent replicas of the workload: the only collectives are the
    barriers around the timed region and the reductions of its results."""
    import torch
    import torch.distributed as dist

    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)


def _reduce_over_ranks(x, op, world, device="cuda"):
    """``x`` reduced over all ranks: op "max" (the elapsed times: the job ends
    with its slowest rank) or "sum" (the particles every rank processed)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t)


def _barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def job_throughput(units_per_rank, elapsed, world, device="cuda"):
    """Whole-job units/s: the units of all ranks over the slowest rank's time."""
    return (_reduce_over_ranks(units_per_rank, "sum", world, device)
            / _reduce_over_ranks(elapsed, "max", world, device))


def movers_fraction(p, torch):
    """Fraction of live particles outside their cell (after an advection!)."""
    idx = p.index.data.bool()
    live = int(idx.sum())
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
    return int((out & idx).sum()) / max(1, live)


L2_BYTES = 129e6


def l2_policy(cfg, f32=False):
    """(flush, note): the particle arrays (coordinates or offsets, fields,
    occupancy bytes over every slot) against GB300's 129 MB L2. Below twice its
    size a 256 MB buffer is written before every timed step, outside the
    timing, so that no step starts with its inputs in L2."""
    ni = cfg["grid"]["ni"]
    N = len(ni)
    nf = cfg.get("fields", 0)
    vb = 4 if f32 else 8
    b = float(np.prod(ni)) * cfg["max_xcell"] * ((N + nf) * vb + 1)
    if b > 2 * L2_BYTES:
        return False, f"inputs larger than L2: the particle arrays are {b / 1e6:.0f} MB against 129 MB"
    return True, (f"the particle arrays ({b / 1e6:.0f} MB) fit the 129 MB L2: a 256 MB buffer is written "
                  "before every timed step, outside the timing")


def workload_config(args, f32=False):
    """The ``config`` object of a bench line: what defines the workload, the
    same in this arm and in the reference arm."""
    cfg = _setup_cfg(args.workload, args.ni)
    rk4 = args.method == "rk4" or (args.method is None and cfg["method"] == "RK4")
    desc = DESC[args.workload] if args.ni is None else DESC[args.workload] + f" (resized to {args.ni} cells per axis)"
    return {
        "workload": desc,
        "form": "split precision (FP32 cell offset)" if f32 else "FP64",
        "integrator": "RungeKutta4" if rk4 else "RungeKutta2",
        "cells": list(cfg["grid"]["ni"]),
        "particles_per_cell": [cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"]],
        "dt": cfg["dt"],
        "l2": l2_policy(cfg, f32)[1],
    }


def _setup_cfg(workload, ni):
    from justpic_gb300 import workloads as W
    base = W.CONFIGS[workload]["ni"]
    return W.setup(workload, None if ni is None else (ni,) * len(base))


def run_ours(args, form=None, minimal=False):
    """The bench line. With ``minimal`` (used for the split-precision figures
    added to the FP64 line) only the device-resident timing is done and the
    result is returned instead of printed."""
    import torch

    import justpic_gb300 as jp

    world, rank, local = _dist()
    if world > 1 and not minimal:
        _init_ranks(local)
    elif world == 1:
        torch.cuda.set_device(0)
    jp._native.load()

    cfg = _setup_cfg(args.workload, args.ni)
    g = cfg["grid"]
    N = g["ndim"]
    nf = 1 if "particle2grid!" in STEPS[args.workload] else 0
    dt = cfg["dt"]
    f32 = (form or args.form) == "f32"
    p = jp.init_particles(jp.CUDABackend, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], *g["grid_v"],
                          seed=jp.DEFAULT_SEED + rank)
    V = tuple(jp.TA("CUDA")(v) for v in cfg["V"])
    T = jp.TA("CUDA")(cfg["T"])
    if f32:
        xi = jp.init_offsets(p)
        fields = jp.init_cell_arrays_f32(p, nf)
        V = tuple(v.float() for v in V)
        T = T.float()
    else:
        fields = jp.init_cell_arrays(p, nf)
    pT = fields[0] if nf else None
    rk4 = args.method == "rk4" or (args.method is None and cfg["method"] == "RK4")
    method = jp.RungeKutta4() if rk4 else jp.RungeKutta2()

    stream = torch.cuda.current_stream()
    ops = STEPS[args.workload]
    Vcur = [V]

    def call(op):
        if f32:
            if op == "particle2grid!":
                jp.particle2grid_f32_(T, pT, p, xi)
            elif op == "advection!":
                jp.advection_f32_(p, xi, method, Vcur[0], dt)
            elif op == "move_particles!":
                jp.move_particles_f32_(p, xi, fields)
            elif op == "inject_particles!":
                jp.inject_particles_f32_(p, xi, fields)
            elif op == "grid2particle!":
                jp.grid2particle_f32_(pT, T, p, xi)
            return
        if op == "particle2grid!":
            jp.particle2grid_(T, pT, p)
        elif op == "advection!":
            jp.advection_(p, method, Vcur[0], dt)
        elif op == "move_particles!":
            jp.move_particles_(p, fields)
        elif op == "inject_particles!":
            jp.inject_particles_(p, fields)
        elif op == "grid2particle!":
            jp.grid2particle_(pT, T, p)

    def step(ev=None):
        for k, op in enumerate(ops):
            if ev is not None:
                ev[k][0].record(stream)
            call(op)
            if ev is not None:
                ev[k][1].record(stream)

    if nf:
        call("grid2particle!")
    # movers fraction of this workload (measured once, outside the timed region)
    if nf:
        call("particle2grid!")
    call("advection!")
    if f32:
        live_mask = p.index.data.bool()
        out = torch.zeros_like(live_mask)
        for d in range(N):
            x = xi[d].data
            out |= ~((x >= 0) & (x < 1))
        m = int((out & live_mask).sum()) / max(1, int(live_mask.sum()))
    else:
        m = movers_fraction(p, torch)
    call("move_particles!")
    if "inject_particles!" in ops:
        call("inject_particles!")
    if "grid2particle!" in ops:
        call("grid2particle!")

    # ---- device-resident throughput (asynchronous calls) ----
    jp.set_synchronous(p, False)
    for _ in range(args.warmup):
        step()
    jp.synchronize(p)
    jp.move_counts(p, clear=True)
    live0 = int(p.index.data.sum())
    events = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)] for _ in ops]
              for _ in range(args.steps)]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush = l2_policy(cfg, f32)[0]
    scrub = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if flush else None
    _barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0.record(stream)
        for k in range(args.steps):
            if scrub is not None:  # evict the step's inputs from L2 (not timed: per-step events below)
                scrub.fill_(k & 0xFF)
            step(events[k])
        t1.record(stream)
        torch.cuda.synchronize()
    jp.synchronize(p)
    _barrier(world)
    removed = jp.move_counts(p, clear=True)
    live1 = int(p.index.data.sum())
    live = 0.5 * (live0 + live1)
    if scrub is not None:  # the steps alone, without the flushes between them
        elapsed_rank = sum(events[k][0][0].elapsed_time(events[k][-1][1]) for k in range(args.steps)) / 1e3
    else:
        elapsed_rank = t0.elapsed_time(t1) / 1e3
    elapsed = _reduce_over_ranks(elapsed_rank, "max", world)
    value = job_throughput(live * args.steps, elapsed_rank, world)
    op_ms = {op: float(np.mean([events[k][i][0].elapsed_time(events[k][i][1]) for k in range(args.steps)]))
             for i, op in enumerate(ops)}
    # ---- roofline of the dominant call ----
    peak, peak_kind = _peaks()
    nvel_bytes = sum(v.size * 8 for v in cfg["V"])
    slots_per_live = p.max_xcell * int(np.prod(p.ni)) / live
    gb = nvel_bytes / live
    fb = T.numel() * 8 / live
    vb = 4 if f32 else 8  # bytes per value of coordinates/offsets and fields
    bpp = {op: algorithmic_bytes(op, N, nf, m, slots_per_live, gb * vb / 8, fb * vb / 8, vb) for op in ops}
    dom = max(op_ms, key=op_ms.get)
    achieved = bpp[dom] * live / (op_ms[dom] / 1e3) / 1e9
    step_bytes = sum(bpp.values()) * live
    step_gbs = step_bytes / (elapsed / args.steps) / 1e9
    traffic_table = DRAM_BYTES_PER_PARTICLE.get(("C2" if args.workload == "C4" else args.workload,
                                                 "f32" if f32 else "f64"), {})
    roofline = {
        "bound": "hbm",
        "kernel": dom,
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
        "peak_source": "measured hbm_gbs (MEASURED_PEAKS.json)" if peak_kind == "measured"
        else "fallback 6.8 TB/s",
        "traffic": traffic_table[dom] * live / 1e9 if dom in traffic_table else None,
        "traffic_unit": "GB per call, from an ncu capture of the workload at its own size (C4: of C2), "
                        "bytes per particle x this run's live particles",
        "per_call_frac": {op: bpp[op] * live / (op_ms[op] / 1e3) / 1e9 / peak for op in ops},
    }
    if minimal:
        return {"value": value, "ms_per_step": 1e3 * elapsed / args.steps,
                "per_call_ms": op_ms, "clocks": clocks.summary(), "move_removed": removed,
                "algorithmic_bytes_per_particle": bpp, "step_algorithmic_gbs": step_gbs, "roofline": roofline}

    # ---- end to end through the public API (synchronous, host buffers) ----
    jp.set_synchronous(p, True)
    hdt = np.float32 if f32 else np.float64
    hV = [torch.from_numpy(np.ascontiguousarray(v.transpose(tuple(reversed(range(v.ndim)))), dtype=hdt)).pin_memory()
          for v in cfg["V"]]
    dV = [torch.empty_like(h, device="cuda") for h in hV]
    rev = tuple(reversed(range(N)))
    hT = torch.empty(tuple(reversed(T.shape)), dtype=T.dtype).pin_memory() if nf else None
    e2e_steps = max(1, min(args.steps, 50))
    _barrier(world)
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    e2e_time = 0.0
    for k in range(e2e_steps):
        if scrub is not None:  # as above: L2 flushed before each step, outside the timing
            scrub.fill_(k & 0xFF)
            torch.cuda.synchronize()
            w0 = time.perf_counter()
        for h, d in zip(hV, dV):
            d.copy_(h, non_blocking=True)
        Vcur[0] = tuple(d.permute(*rev) for d in dV)
        step()
        if nf:
            hT.copy_(T.permute(*rev), non_blocking=False)
        if scrub is not None:
            torch.cuda.synchronize()
            e2e_time += time.perf_counter() - w0
    torch.cuda.synchronize()
    if scrub is None:
        e2e_time = time.perf_counter() - w0
    Vcur[0] = V
    e2e_value = job_throughput(live * e2e_steps, e2e_time, world)

    # the interpolating kernels are bound by GB300's FP64 issue rate (2 lanes per clock
    # per SM), not by HBM: their FP64 instruction rate against that peak at the sampled clock
    fp64_roof = None
    fi = fp64_instructions(dom, N, type(method).__name__) if not f32 else None
    if fi is not None:
        mhz = clocks.summary().get("sm_mhz") or 2070.0
        peak_i = 152 * 2 * mhz * 1e6
        ach_i = fi * live / (op_ms[dom] / 1e3)
        fp64_roof = {"kernel": dom, "fp64_instructions_per_particle": fi, "achieved_ginst_s": ach_i / 1e9,
                     "peak_ginst_s": peak_i / 1e9, "frac": ach_i / peak_i,
                     "peak_source": "152 SMs x 2 FP64 lanes per clock x sampled SM clock"}

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
        "dtype": "f32 offsets + int32 cell (FP64 renormalisation and p2g sums)" if f32 else "f64",
        "data": "synthetic (seeded analytic flow; the reference publishes no dataset)",
        "config": workload_config(args, f32),
        "workload_stats": {"live_particles": live, "movers_fraction": m,
                           "parallelism": "independent replicas" if world > 1 else "single GPU"},
        "per_call_ms": op_ms,
        "algorithmic_bytes_per_particle": bpp,
        "step_algorithmic_gbs": step_gbs,
        "fp64_roofline": fp64_roof,
        "roofline": roofline,
        "e2e": {
            "value": e2e_value,
            "unit": UNIT,
            "h2d_bytes_per_step": int(sum(h.numel() * h.element_size() for h in hV)),
            "d2h_bytes_per_step": int(hT.numel() * hT.element_size()) if nf else 0,
            "steps": e2e_steps,
            "mode": "public API, synchronous calls; velocity grids in and (with fields) the vertex field out each step",
        },
        "gpu_launches": sum(launches(op, N) for op in ops) * args.steps,
        "move_removed": dict(removed, steps=args.steps,
                             note="particles move_particles! removed over the timed steps: left the domain, moved "
                                  "more than one cell (dropped), no free slot in the new cell (dropped)"),
        "clocks": clocks.summary(),
    }
    if not f32 and N == 2 and not args.no_split:
        # the split-precision form on the same workload, and its error against this form
        del p, fields, pT
        sp = run_ours(args, "f32", True)
        sp["speedup_vs_fp64"] = sp["value"] / value
        sp["form"] = "split precision: int32 cell + FP32 offset, FP32 velocities/fields, FP64 renormalisation " \
                     "and particle2grid! sums"
        if rank == 0:
            cmp_steps = 100
            sp["error_vs_fp64"] = run_compare(args, steps=cmp_steps, quiet=True)
        result["split_precision"] = sp
    if rank == 0 and world == 1 and args.workload == "C2" and args.ni is None and not args.no_extra:
        result.update(run_c4_c5(args))
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args.workload, args.cpu_seconds)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(result))


def run_compare(args, steps=None, quiet=False):
    """The same seeded run in both forms for ``--steps`` steps (no timing):
    position error of the split-precision form in cell widths, by particle id,
    for every initial particle still present in both runs (injected particles
    copy a neighbour's fields, so their ids are cleared), and L-inf / L2 error
    of the gridded field, both against the FP64 form."""
    import torch

    import justpic_gb300 as jp

    if not quiet:
        torch.cuda.set_device(0)
    nsteps = steps or args.steps
    cfg = _setup_cfg(args.workload, args.ni)
    g = cfg["grid"]
    N = g["ndim"]
    dt = cfg["dt"]
    rk4 = args.method == "rk4" or (args.method is None and cfg["method"] == "RK4")
    method = jp.RungeKutta4() if rk4 else jp.RungeKutta2()
    a = jp.init_particles(jp.CUDABackend, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], *g["grid_v"])
    b = jp.init_particles(jp.CUDABackend, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], *g["grid_v"])
    live = a.index.data.bool()
    ids = torch.full(a.index.data.shape, float("nan"), dtype=torch.float64, device="cuda")
    ids[live] = torch.arange(int(live.sum()), device="cuda", dtype=torch.float64)
    hi = torch.floor(ids / 4096.0)
    lo = ids - hi * 4096.0
    Ta = jp.TA("CUDA")(cfg["T"])
    Tb = Ta.float()
    Va = tuple(jp.TA("CUDA")(v) for v in cfg["V"])
    Vb = tuple(v.float() for v in Va)
    pTa, = jp.init_cell_arrays(a, 1)
    pTb, = jp.init_cell_arrays_f32(b, 1)
    fa = (pTa, jp.CellArray(ids, a.ni))
    fb = (pTb, jp.CellArray(hi.float().contiguous(), b.ni), jp.CellArray(lo.float().contiguous(), b.ni))
    xi = jp.init_offsets(b)
    jp.set_synchronous(a, False)
    jp.set_synchronous(b, False)
    jp.grid2particle_(pTa, Ta, a)
    jp.grid2particle_f32_(pTb, Tb, b, xi)
    w0 = time.perf_counter()
    for _ in range(nsteps):
        jp.particle2grid_(Ta, pTa, a)
        jp.advection_(a, method, Va, dt)
        jp.move_particles_(a, fa)
        before = a.index.data.clone()
        jp.inject_particles_(a, fa)
        fa[1].data[a.index.data.bool() & ~before.bool()] = float("nan")  # injected copies carry no id
        jp.grid2particle_(pTa, Ta, a)
        jp.particle2grid_f32_(Tb, pTb, b, xi)
        jp.advection_f32_(b, xi, method, Vb, dt)
        jp.move_particles_f32_(b, xi, fb)
        before = b.index.data.clone()
        jp.inject_particles_f32_(b, xi, fb)
        new = b.index.data.bool() & ~before.bool()
        fb[1].data[new] = float("nan")
        fb[2].data[new] = float("nan")
        jp.grid2particle_f32_(pTb, Tb, b, xi)
    jp.synchronize(a)
    jp.synchronize(b)
    wall = time.perf_counter() - w0
    # original particles only: every injected particle (and its copies' ids) was marked NaN
    la = a.index.data.bool() & ~torch.isnan(fa[1].data)
    lb = b.index.data.bool() & ~torch.isnan(fb[1].data)
    ida = fa[1].data[la].long()
    idb = (fb[1].data[lb].double() * 4096 + fb[2].data[lb].double()).long()
    pa = torch.stack([c.data[la] for c in a.coords], 1)
    back = jp.coords_from_offsets(b, xi)
    pb = torch.stack([c.data[lb] for c in back], 1)
    n_ids = int(max(int(ida.max()), int(idb.max()))) + 2

    def unique_pos(idv, pos):
        cnt = torch.bincount(idv, minlength=n_ids)
        keep = cnt[idv] == 1
        table = torch.full((n_ids, N), float("nan"), dtype=torch.float64, device="cuda")
        table[idv[keep]] = pos[keep]
        return table

    ta, tb = unique_pos(ida, pa), unique_pos(idb, pb)
    both = ~torch.isnan(ta[:, 0]) & ~torch.isnan(tb[:, 0])
    dxs = torch.tensor(g["dx"], dtype=torch.float64, device="cuda")
    err = ((ta[both] - tb[both]).abs() / dxs).max(dim=1).values
    Ferr = (Ta.double() - Tb.double())
    out = {
        "workload": DESC[args.workload] if args.ni is None else DESC[args.workload] + f" (resized to {args.ni})",
        "integrator": type(method).__name__,
        "steps": nsteps,
        "particles_compared": int(both.sum()),
        "live_fp64": int(a.index.data.sum()), "live_split": int(b.index.data.sum()),
        "position_error_cells": {"max": float(err.max()), "p99": float(torch.quantile(err[:1 << 24], 0.99)),
                                 "mean": float(err.mean())},
        "gridded_field_error": {"linf": float(Ferr.abs().max()),
                                "l2_rel": float(Ferr.norm() / Ta.norm()),
                                "field_range": float(Ta.max() - Ta.min())},
        "wall_s_both_forms": wall,
    }
    if quiet:
        return out
    print(json.dumps(out))


def run_adjoint(args, quiet=False):
    """C5: cost of the checkpointed gradient against the forward run alone,
    and central finite differences (h = 1e-6) on --fd-nodes random velocity
    nodes, each formed vertex by vertex. Printed, or returned when ``quiet``."""
    import torch

    import justpic_gb300 as jp
    from justpic_gb300 import adjoint as A

    torch.cuda.set_device(0)
    cfg = _setup_cfg("C5", args.ni)
    g = cfg["grid"]
    nsteps = args.adjoint_steps or cfg["steps"]
    k = cfg["checkpoint_every"]
    p = jp.init_particles(jp.CUDABackend, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], *g["grid_v"])
    V = tuple(jp.TA("CUDA")(v) for v in cfg["V"])
    dt = cfg["dt"]
    (T0,) = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(T0, jp.TA("CUDA")(cfg["T"]), p)
    target = jp.TA("CUDA")(cfg["T_target"])
    method = jp.RungeKutta2()
    live = int(p.index.data.sum())

    def timed(fn, reps):
        ts = []
        out = None
        for _ in range(reps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            out = fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return float(np.median(ts)), out

    fwd = lambda: A.forward_field(p, method, V, dt, nsteps, T0)  # noqa: E731
    kept = A.kept_segments(p, method, nsteps, k)
    grad = lambda: A.misfit_gradient(p, method, V, dt, nsteps, T0, target, checkpoint_every=k)  # noqa: E731
    grad1 = lambda: A.misfit_gradient(p, method, V, dt, nsteps, T0, target, checkpoint_every=k,  # noqa: E731
                                      record_segments=1)
    if args.form == "f32":  # the split-precision variant on the same run
        xi = jp.init_offsets(p)
        V32 = tuple(v.float() for v in V)
        T0f = jp.CellArray(T0.data.float().contiguous(), p.ni)
        tgt32 = target.float()

        def fwd():
            st = A._save_f32(p, xi)
            T = jp.CellArray(T0f.data.clone(), p.ni)
            try:
                for _ in range(nsteps):
                    jp.advection_f32_(p, xi, method, V32, dt)
                    jp.move_particles_f32_(p, xi, (T,))
                    jp.inject_particles_f32_(p, xi, (T,))
                F = jp.grid_field_f32(tuple(n + 1 for n in p.ni))
                jp.particle2grid_f32_(F, T, p, xi)
            finally:
                A._restore_f32(p, xi, st)

        grad = lambda: A.misfit_gradient_f32(p, xi, method, V32, dt, nsteps, T0f, tgt32,  # noqa: E731
                                             checkpoint_every=k)
        grad1 = lambda: A.misfit_gradient_f32(p, xi, method, V32, dt, nsteps, T0f, tgt32,  # noqa: E731
                                              checkpoint_every=k, record_segments=1)
        kept = A.kept_segments_f32(p, nsteps, k)
    for _ in range(max(1, min(args.warmup, 3))):
        fwd()
        grad()
    reps = max(1, min(args.steps, 5))
    t_fwd, _ = timed(fwd, reps)
    t_grad, (loss, gV, gT0) = timed(grad, reps)
    grad1()
    t_grad1, _ = timed(grad1, reps)
    rng = np.random.default_rng(17)
    checked = []
    h = 1e-6
    Vh = cfg["V"]
    gmax = max(float(gv.abs().max()) for gv in gV)
    for n in range(args.fd_nodes if args.form == "f64" else 0):
        # even n: any node; odd n: a node where |dL/dV| is at least 1e-3 of its maximum
        c = (n // 2) % 2
        gc = gV[c].cpu().numpy()
        flat = gc.reshape(-1, order="F")
        pool = np.flatnonzero(np.abs(flat) >= 1e-3 * gmax) if n % 2 else np.arange(flat.size)
        node = np.unravel_index(int(rng.choice(pool)), gc.shape, order="F")
        Vp = [v.copy(order="F") for v in Vh]
        Vm = [v.copy(order="F") for v in Vh]
        Vp[c][node] += h
        Vm[c][node] -= h
        Fp, Wp = A.forward_field(p, method, tuple(jp.TA("CUDA")(v) for v in Vp), dt, nsteps, T0)
        Fm, Wm = A.forward_field(p, method, tuple(jp.TA("CUDA")(v) for v in Vm), dt, nsteps, T0)
        fd = A.misfit_difference(Fp, Wp, Fm, Wm, target) / (2 * h)
        checked.append((float(gc[node]), fd))
    fd_out = {"nodes": len(checked), "h": h}
    if checked:
        adj = np.array([a for a, _ in checked])
        fd = np.array([f for _, f in checked])
        err = np.abs(adj - fd)
        active = np.abs(fd) >= 1e-3 * gmax
        fd_out.update({
            "max_err_over_max_gradient": float(np.max(err) / gmax),
            "max_rel_err_active_nodes": float(np.max(err[active] / np.abs(fd[active]))) if active.any() else None,
            "active_nodes": int(active.sum()),
            "active": "|fd| >= 1e-3 of max |dL/dV|",
            "pairs_adjoint_fd": [[float(a), float(f)] for a, f in checked[:8]],
        })
    pbytes = float(np.prod(cfg["grid"]["ni"])) * cfg["max_xcell"] * (3 * (4 if args.form == "f32" else 8) + 1)
    out = {
        "form": "split precision (FP32 offsets, FP64 cotangents)" if args.form == "f32" else "FP64",
        "workload": DESC["C5"] if args.ni is None else DESC["C5"] + f" (resized to {args.ni})",
        "live_particles": live, "steps": nsteps, "checkpoint_every": k, "loss": loss,
        "forward_s": t_fwd, "forward_plus_gradient_s": t_grad, "gradient_cost_vs_forward": t_grad / t_fwd,
        "records_kept_segments": kept,
        "records": "checkpoints every checkpoint_every steps; the records of the last records_kept_segments "
                   "segments stay in HBM (budget 64 GB), every other segment is run again from its checkpoint",
        "gradient_cost_vs_forward_one_segment_kept": t_grad1 / t_fwd,
        "forward_particle_steps_per_s": live * nsteps / t_fwd,
        "l2": f"whole runs timed: every step streams the particle arrays ({pbytes / 1e6:.0f} MB), and the "
              "gradient run its stage records (GBs), through the 129 MB L2",
        "max_abs_gradient": gmax,
        "fd_check": fd_out,
    }
    if quiet:
        return out
    print(json.dumps(out))


def run_c4_c5(args):
    """The figures of the other two GPU configurations, added to the default
    line: C4 (2048^2, RK4, both forms, a short timed window each, and the
    position error of the split form after 750 RK2 steps of the miniapp cycle
    against the FP64 form) and C5 (the adjoint's cost against its forward run,
    FP64 and FP32 variants)."""
    import torch

    c4 = argparse.Namespace(**vars(args))
    c4.workload, c4.ni, c4.method, c4.steps, c4.warmup = "C4", None, None, 10, 3
    f64 = run_ours(c4, "f64", True)
    torch.cuda.empty_cache()
    f32 = run_ours(c4, "f32", True)
    torch.cuda.empty_cache()
    rk2 = argparse.Namespace(**vars(c4))
    rk2.method = "rk2"
    err = run_compare(rk2, steps=750, quiet=True)
    torch.cuda.empty_cache()
    out = {"C4": {
        "workload": DESC["C4"],
        "timed_steps": c4.steps,
        "fp64": {k: f64[k] for k in ("value", "ms_per_step", "per_call_ms", "roofline")},
        "split": {k: f32[k] for k in ("value", "ms_per_step", "per_call_ms", "roofline")},
        "speedup_split_vs_fp64": f32["value"] / f64["value"],
        "error_after_750_rk2_steps": err,
    }}
    c5 = argparse.Namespace(**vars(args))
    c5.workload, c5.ni, c5.adjoint_steps, c5.fd_nodes, c5.steps, c5.warmup = "C5", None, 0, 0, 5, 3
    keys = ("forward_s", "forward_plus_gradient_s", "gradient_cost_vs_forward",
            "gradient_cost_vs_forward_one_segment_kept", "records_kept_segments", "live_particles", "steps",
            "checkpoint_every")
    c5.form = "f64"
    a64 = run_adjoint(c5, quiet=True)
    torch.cuda.empty_cache()
    c5.form = "f32"
    a32 = run_adjoint(c5, quiet=True)
    torch.cuda.empty_cache()
    out["C5"] = {"workload": DESC["C5"], "fp64": {k: a64[k] for k in keys}, "fp32": {k: a32[k] for k in keys}}
    return out


def _cpu_setup(workload):
    from oracle import oracle as O

    cfg = _setup_cfg(workload, None)
    g = cfg["grid"]
    ops = STEPS[workload]
    nf = 1 if "particle2grid!" in ops else 0
    grids = tuple(tuple(np.asarray(x) for x in comp) for comp in g["grid_v"])
    o = O.OracleParticles(grids, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], uniform=True)
    o.init_particles()
    fields = [o.cell_array() for _ in range(nf)]
    T = np.asfortranarray(cfg["T"].copy())
    if nf:
        o.grid2particle(fields[0], T)
    V = cfg["V"]
    dt = cfg["dt"]

    def step():
        for op in ops:
            if op == "particle2grid!":
                o.particle2grid(T, fields[0])
            elif op == "advection!":
                o.advection(O.RK4 if cfg["method"] == "RK4" else O.RK2, 0.5, V, dt)
            elif op == "move_particles!":
                o.move_particles(fields)
            elif op == "inject_particles!":
                o.inject_particles(fields)
            elif op == "grid2particle!":
                o.grid2particle(fields[0], T)

    return o, step


def cpu_baseline(workload="C2", seconds=20.0, max_steps=None):
    """The FP64 C restatement of the reference's CPU path, all host threads, on
    the same workload; times whole steps until ``seconds`` of CPU work."""
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    O.set_threads(cores)
    o, step = _cpu_setup(workload)
    step()  # warm-up (page faults, thread pool)
    n, t, live_sum = 0, 0.0, 0
    while t < seconds and (max_steps is None or n < max_steps):
        live_sum += int(o.index.sum())
        w0 = time.perf_counter()
        step()
        t += time.perf_counter() - w0
        n += 1
    return {"value": live_sum / t, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} full {workload} steps in {t:.1f} s with {cores} OpenMP threads; FP64 C restatement of "
                      "the reference's CPU path (Julia is not available)"}


def run_reference(args):
    world, rank, _ = _dist()
    if rank != 0:
        return
    from oracle import oracle as O

    cores = os.cpu_count() or 1
    O.set_threads(cores)
    o, step = _cpu_setup(args.workload)
    for _ in range(max(0, min(args.warmup, 1))):
        step()
    budget = 90.0
    n, t, live_sum = 0, 0.0, 0
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
        "data": "synthetic (seeded analytic flow; the reference publishes no dataset)",
        "config": workload_config(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{n} of {args.steps} requested full steps timed (capped at {budget:.0f} s); "
                                   "FP64 C restatement of JustPIC's CPU path (Julia is not installed)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(STEPS), default="C2")
    ap.add_argument("--form", choices=["f64", "f32"], default="f64",
                    help="f64: the reference's FP64 form; f32: int32 cell + FP32 offset form")
    ap.add_argument("--method", choices=["rk2", "rk4"], default=None,
                    help="integrator (default: the workload's, RK2 except C4)")
    ap.add_argument("--compare-forms", action="store_true",
                    help="run the same seeded workload in both forms for --steps steps and print the errors")
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-split", action="store_true",
                    help="FP64 line without the split-precision timing and error added to it")
    ap.add_argument("--no-extra", action="store_true",
                    help="default line without the C4 (both forms) and C5 (adjoint) figures")
    ap.add_argument("--adjoint-steps", type=int, default=0,
                    help="C5: steps of the run (default: the workload's 100)")
    ap.add_argument("--fd-nodes", type=int, default=0,
                    help="C5: number of random velocity nodes checked by central finite differences")
    ap.add_argument("--ni", type=int, default=None,
                    help="cells per axis instead of the workload's (small cases for ncu captures; not a bench line)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.workload == "C5" and args.impl == "ours":
        run_adjoint(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.compare_forms:
        run_compare(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
