#!/usr/bin/env python
"""Benchmark: steady-state I-V points per second of the PECS half cell on GB300.

Workload: the coupled semiconductor--electrolyte half cell, semiconductor
[0,1]^2 and electrolyte [1,2]x[0,1], 64x64 cells each (refinement 6), LDG
degree 1, mixed RT_0 x DGQ_0 Poisson (the reference's RT_{k-1} x DGQ_{k-1}
pairing), dt = 1e-3.  One I-V point = one parameter draw (bias, generation,
absorption, doping, lifetimes, interface rates) marched until the relative
change of every field is <= 1e-8 or 5000 steps.  Inputs are synthetic (no
dataset exists for this model): seeded parameter draws.

Default (full) mode, one bench step = 64 held-out points:
  value   learned + batched: the points streamed through 64 slots of one
          context in FP32-mixed precision with increment solves (one FP32
          sweep per solve on the residual against the previous step; the
          same fixed point as refined solves), each warm-started by the neural
          operator (first-step-residual fallback), timed with CUDA events on
          the library's stream, parameters uploaded per refill, L2 flushed.
  e2e     64 further points through the public C ABI (pecs_sweep_stream) with
          host parameters in and currents and all final fields out.
  plain   beside it: one point on the plain single-instance FP64 path, and
          the same points batched without the warm start.
--mode plain times the plain path alone (one bench step = one point).

--impl reference times the CPU oracle (the restatement of the reference's
numerics; the deal.II reference itself cannot be built here): one oracle
process per host core, each marching the plain point's time steps from the
standard initial condition; every bench step is `--cpu-sample-steps` IMEX
steps of every process, timed together, and `ms_per_step` is that measured
time.  Points/sec is derived from the measured time per IMEX step and the
plain point's steps to steady state (`profiles/steps_to_steady_state.json`,
measured on the GPU's plain FP64 path, which marches the same discrete
scheme).

Multi-GPU: I-V points are independent, so each rank marches its own instances
(weak scaling, no data-path collective); the barrier and max-over-ranks time
use torch.distributed.
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
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

MAX_STEPS = 5000
TOL = 1e-8
CHECK_EVERY = 50
L2_FLUSH_BYTES = 512 << 20   # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--refine", type=int, default=6)
    ap.add_argument("--precision", choices=["fp64", "fp32ir", "mixed"], default="fp64")
    ap.add_argument("--n-inst", type=int, default=1, help="instances per GPU per bench step")
    ap.add_argument("--cpu-sample-steps", type=int, default=8,
                    help="IMEX steps of every oracle process per bench step of --impl reference")
    ap.add_argument("--ref-procs", type=int, default=0,
                    help="--impl reference: oracle processes (0 = one per host core)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", choices=["full", "plain", "ragged"], default="full",
                    help="full: learned warm start + 64-instance batches (FP32-mixed) with the "
                         "plain FP64 path measured beside it; plain: one configuration only; "
                         "ragged: 64 instances of refinement 5-7 and degree 1-2 (--precision, "
                         "default FP64), one context per mesh group")
    ap.add_argument("--batch-inst", type=int, default=64)
    ap.add_argument("--concurrent", type=int, choices=[0, 1], default=0,
                    help="ragged mode: run the mesh groups' sweeps at the same time (one host "
                         "thread and CUDA stream per group) instead of one after another")
    ap.add_argument("--leaf-cells", type=int, default=8,
                    help="nested-dissection leaf size in cells (the solve tree's height)")
    ap.add_argument("--increment", type=int, choices=[0, 1], default=1,
                    help="mixed precision: time steps solve for the increment from the previous "
                         "step (one FP32 sweep per solve, same fixed point); 0 = refined solves")
    ap.add_argument("--flow", type=int, choices=[-1, 0, 1], default=0,
                    help="batched solve sweeps: 1 = one persistent launch per direction, "
                         "-1 = one launch per tree level, 0 = whichever the autotuner times faster")
    ap.add_argument("--e2e-waves", type=int, default=4,
                    help="full mode: end-to-end points = this many times --batch-inst")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="full mode: skip the FP64 accuracy references (profiling runs)")
    ap.add_argument("--model", default=os.path.join(ROOT, "pecs_gb300", "models", "warmstart_ref6.npz"))
    ap.add_argument("--train-samples", type=int, default=256,
                    help="training draws when no trained model file is present")
    ap.add_argument("--steady", action="store_true",
                    help="profiler mode: also run once to steady state and list the steps")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="profiler mode: initialise the workload, run this many time steps "
                         "with direct (non-graph) launches, print one line and exit")
    ap.add_argument("--level-times", action="store_true",
                    help="with --profile-sweep (FP32 sweeps): also time every level of the sweep")
    ap.add_argument("--profile-sweep", choices=["carrier", "poisson"], default=None,
                    help="profiler mode: build the workload and run exactly two solve sweeps of "
                         "one bank (a warm-up and a timed one), print one line and exit")
    return ap.parse_args()


def check_world(args):
    """--gpus N must match the launcher's world size (torchrun for N > 1)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world != args.gpus:
        sys.stderr.write(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}; launch N > 1 with "
                         f"torchrun --nproc-per-node N bench.py --gpus N\n")
        sys.exit(2)
    return world


def dist_init(args):
    import torch
    world = check_world(args)
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def load_traffic(key: str):
    """Per-launch DRAM bytes from the committed ncu summary (profiles/), or None."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as fh:
            return json.load(fh).get(key)
    except (OSError, ValueError):
        return None


def load_steps_to_ss(refine: int):
    """Steps to steady state of the plain point (half cell, standard initial
    condition, FP64) at this refinement, measured by this benchmark on the GPU
    (profiles/steps_to_steady_state.json), or None."""
    p = os.path.join(ROOT, "profiles", "steps_to_steady_state.json")
    try:
        with open(p) as fh:
            return int(json.load(fh)["steps"][str(refine)])
    except (OSError, KeyError, ValueError):
        return None


def workload_params(args, rank):
    import pecs_gb300 as pg
    n = args.n_inst
    ps = []
    for i in range(n):
        # each rank/instance one point of an I-V sweep (bias in thermal-voltage units)
        g = rank * n + i
        bias = 0.0 if n == 1 else -0.5 + (g % 64) / 63.0
        ps.append(pg.half_cell(n_refine=args.refine, phi_app=bias))
    return ps


def _reference_worker(refine, n_samples, sample_steps, barrier, out):
    """One oracle process: builds the problem and its LU factors (untimed),
    then marches the plain point from its standard initial condition, timing
    `n_samples` samples of `sample_steps` IMEX steps, each sample started
    together with the other processes at the barrier."""
    import oracle
    pb = oracle.Problem(oracle.half_cell_params(n_refine=refine))
    st = pb.step(pb.initial_state())   # the first step builds the factors
    per = []
    for _ in range(n_samples):
        barrier.wait()
        t0 = time.perf_counter()
        for _ in range(sample_steps):
            st = pb.step(st)
        per.append(time.perf_counter() - t0)
    out.put(per)


def oracle_pool(refine, n_samples, sample_steps, procs):
    """`procs` oracle processes (spawned; BLAS single-threaded), each timing
    n_samples samples of sample_steps IMEX steps.  Returns (per-process
    lists of sample seconds, wall seconds of each sample: the slowest
    process's, since the samples start together)."""
    import multiprocessing as mp
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[var] = "1"
    ctx = mp.get_context("spawn")
    bar = ctx.Barrier(procs)
    out = ctx.Queue()
    ps = [ctx.Process(target=_reference_worker, args=(refine, n_samples, sample_steps, bar, out))
          for _ in range(procs)]
    for p in ps:
        p.start()
    per = [out.get() for _ in ps]
    for p in ps:
        p.join()
    wall = [max(w[k] for w in per) for k in range(n_samples)]
    return per, wall


def host_cores():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def cpu_baseline(args, steps_to_ss, sample_steps=4, samples=2):
    """The oracle on every host core (one process per core, each marching the
    plain point), a bounded sample of IMEX steps; I-V points/sec from the
    measured time per step and the steps to steady state that the GPU's plain
    FP64 path measured in this run (the same discrete scheme)."""
    procs = host_cores() if args.ref_procs <= 0 else min(host_cores(), args.ref_procs)
    per, wall = oracle_pool(args.refine, samples, sample_steps, procs)
    t_step = statistics.mean(wall) / sample_steps
    return {"value": procs / (steps_to_ss * t_step), "unit": "I-V points/s", "cores": procs, "kind": "port",
            "sample": f"{procs} oracle processes (one per host core), {samples} x {sample_steps} IMEX steps "
                      f"each of the {2**args.refine}x{2**args.refine}+{2**args.refine}x{2**args.refine} "
                      f"half cell ({t_step * 1e3:.1f} ms per step with all cores busy) x {steps_to_ss} "
                      "steps to steady state"}


def run_reference(args):
    world = check_world(args)
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    procs = host_cores() if args.ref_procs <= 0 else min(host_cores(), args.ref_procs)
    per, wall = oracle_pool(args.refine, args.warmup + args.steps, args.cpu_sample_steps, procs)
    timed = wall[args.warmup:]
    ms_step = 1e3 * statistics.mean(timed)                 # one bench step, measured
    t_imex = statistics.mean(timed) / args.cpu_sample_steps
    steps_to_ss = load_steps_to_ss(args.refine)
    source = "measured on the GPU plain FP64 path (profiles/steps_to_steady_state.json)"
    if steps_to_ss is None:
        steps_to_ss, source = MAX_STEPS, "the step cap (no measurement for this mesh)"
    value = procs / (steps_to_ss * t_imex)
    line = {
        "impl": "reference", "metric": "I-V points/sec to steady state", "value": value,
        "unit": "I-V points/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"half cell 2x{2**args.refine}x{2**args.refine}, k=1, dt=1e-3, "
                               f"to steady state (<= {MAX_STEPS} steps)",
                   "bench_step": f"{args.cpu_sample_steps} IMEX steps of each of {procs} oracle processes",
                   "ms_per_imex_step": t_imex * 1e3, "steps_to_steady_state": steps_to_ss,
                   "steps_to_steady_state_source": source,
                   "derived": "value = processes / (steps_to_steady_state x measured time per IMEX step)"},
        "cpu_baseline": {"value": value, "unit": "I-V points/s", "cores": procs, "kind": "port",
                         "sample": f"{procs} oracle processes, each {args.warmup} + {args.steps} x "
                                   f"{args.cpu_sample_steps} IMEX steps of the plain point "
                                   f"({t_imex * 1e3:.1f} ms per step with all cores busy)"},
        "e2e": {"value": value, "unit": "I-V points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_sweep:
        return run_profile_sweep(args)
    if args.mode == "full" and not args.profile_steps:
        return run_full(args)
    if args.mode == "ragged":
        return run_ragged(args)
    return run_plain(args)


def ragged_points(n, seed):
    """Uneven I-V points: refinement uniform on {5, 6, 7}, LDG degree on {1, 2},
    bias U[-0.5, 0.5], G0 U[0.5, 2], alpha U[1, 10], tau log-uniform [0.1, 10]."""
    import numpy as np
    import pecs_gb300 as pg
    rng = np.random.default_rng(seed)
    pts = []
    for _ in range(n):
        tau = float(np.exp(rng.uniform(np.log(0.1), np.log(10.0))))
        pts.append(pg.half_cell(n_refine=int(rng.integers(5, 8)), degree=int(rng.integers(1, 3)),
                                phi_app=float(rng.uniform(-0.5, 0.5)), G0=float(rng.uniform(0.5, 2.0)),
                                alpha=float(rng.uniform(1.0, 10.0)), tau_n=tau, tau_p=tau))
    return pts


def run_ragged(args):
    """64 uneven points per rank to steady state through the public API: the
    points are grouped by mesh and each group is streamed through its own
    context (pecs_sweep_stream), the groups one after another or, with
    --concurrent 1, all at once (one host thread and CUDA stream per group,
    as sweep.ragged_sweep(concurrent=True)); host parameters in, steps and
    currents out.  --precision fp64 (default) or mixed (with --increment).
    One bench step = the 64 points; the contexts' setup (factorisation,
    autotuning) is outside the timed region, as for every other mode (it
    happens once per mesh)."""
    import numpy as np
    import torch
    from concurrent.futures import ThreadPoolExecutor

    import pecs_gb300 as pg
    from pecs_gb300.sweep import matrix_key

    world, rank, local = dist_init(args)
    pg.build()
    n = args.batch_inst
    prec = {"fp64": pg.PREC_FP64, "fp32ir": pg.PREC_FP32_IR, "mixed": pg.PREC_FP32_MIXED}[args.precision]
    groups = {}
    for i, p in enumerate(ragged_points(n * world, 31)[rank * n:(rank + 1) * n]):
        groups.setdefault(matrix_key(p), []).append(p)
    ctxs = [(pts, pg.Context(pts, device=local, precision=prec, increment_solves=bool(args.increment)))
            for pts in groups.values()]
    for pts, c in ctxs:        # warm-up: a few steps of every group
        c.sweep_stream(pts, 3, 1e-30, 3)
    barrier(world)
    torch.cuda.synchronize()
    t0 = 0.0

    def run_group(pc):
        pts, c = pc
        tg = time.perf_counter()
        steps, cur, _ = c.sweep_stream(pts, MAX_STEPS, TOL, CHECK_EVERY)
        p0 = pts[0]
        return {"refine": int(round(np.log2(p0.ny))), "degree": p0.degree, "points": len(pts),
                "seconds": time.perf_counter() - tg, "ends_at_s": time.perf_counter() - t0,
                "median_steps": float(np.median(steps)), "capped": int(np.sum(steps >= MAX_STEPS))}

    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        if args.concurrent:
            with ThreadPoolExecutor(max_workers=len(ctxs)) as pool:
                per_group = list(pool.map(run_group, ctxs))
        else:
            per_group = [run_group(pc) for pc in ctxs]
        torch.cuda.synchronize()
        t_all = time.perf_counter() - t0
    t_all = max_over_ranks(t_all, world)
    if rank == 0:
        mixed = args.precision == "mixed"
        how = ("FP32 factors, increment solves" if mixed and args.increment else
               "FP32 factors, refined solves" if mixed else args.precision.upper())
        line = {"metric": "I-V points/sec to steady state", "value": n * world / t_all,
                "unit": "I-V points/s", "n_gpus": world, "steps": 1, "warmup": 1,
                "ms_per_step": t_all * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+f32-pair" if mixed else "f64", "data": "synthetic",
                "config": {"workload": f"{n} uneven half-cell points per GPU: refinement 5-7, LDG degree 1-2, "
                                       f"{how}, to rel. change <= {TOL} (<= {MAX_STEPS} steps), one context "
                                       "per mesh group, " + ("groups at the same time, one host thread and "
                                                             "stream each" if args.concurrent else
                                                             "groups one after another"),
                           "groups": per_group, "timing": "host wall clock around the public API calls"},
                "clocks": clk.summary()}
        print(json.dumps(line))
    return 0


def run_profile_sweep(args):
    """Two sweeps of one factor bank over the workload's right-hand sides (the
    launches an ncu capture of one sweep selects with -k regex:k_panel or
    regex:"k_forward|k_backward" and -c <launches per sweep>)."""
    import pecs_gb300 as pg
    pg.build()
    prec = {"fp64": pg.PREC_FP64, "fp32ir": pg.PREC_FP32_IR, "mixed": pg.PREC_FP32_MIXED}[args.precision]
    ctx = pg.Context(workload_params(args, 0), precision=prec, leaf_cells=args.leaf_cells,
                     flow_sweep=args.flow, increment_solves=bool(args.increment))
    which = 0 if args.profile_sweep == "carrier" else 1
    info = ctx.info()
    ms = ctx.time_solve(which, reps=1)
    out = {"profile_sweep": args.profile_sweep, "n_inst": args.n_inst, "precision": args.precision,
           "leaf_cells": args.leaf_cells, "factor_entries": list(info.factor_entries),
           "factor_levels": list(info.factor_levels),
           "sweep_ms": ms, "launches_per_sweep": info.solve_launches[which],
           "bytes_per_sweep": info.solve_bytes[which], "launches_setup": info.setup_launches,
           "tuned_sweep_ms": list(info.tuned_sweep_ms), "flow_rpl": list(info.flow_rpl), "flow_top": list(info.flow_top)}
    if args.level_times and args.precision != "fp64" and info.flow_rpl[which] == 0:
        import ctypes as C
        buf = (C.c_double * 64)()
        n = pg.lib().pecs_debug_time_levels(ctx._h, which, 20, buf, 64)
        if n < 0:
            pg._ffi.check(n)
        out["level_ms"] = [round(buf[k], 4) for k in range(n)]
        out["sweep_ms_20"] = ctx.time_solve(which, reps=20)
    print(json.dumps(out))
    return 0


def run_plain(args):
    import numpy as np
    import torch

    import pecs_gb300 as pg

    world, rank, local = dist_init(args)
    pg.build()
    prec = {"fp64": pg.PREC_FP64, "fp32ir": pg.PREC_FP32_IR, "mixed": pg.PREC_FP32_MIXED}[args.precision]
    params = workload_params(args, rank)
    ctx = pg.Context(params, precision=prec, device=local, use_graphs=args.profile_steps == 0,
                     flow_sweep=args.flow, increment_solves=bool(args.increment))
    info = ctx.info()
    if args.profile_steps:
        ctx.initialize()
        ctx.step(3)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.step(args.profile_steps)
        ctx.synchronize()
        ms_step = (time.perf_counter() - t0) * 1e3 / args.profile_steps
        out = {"profile_steps": args.profile_steps, "n_inst": args.n_inst,
               "precision": args.precision, "ms_per_time_step": ms_step,
               "launches_per_step": info.launches_per_step,
               "launches_setup": info.setup_launches,
               "tuned_sweep_ms": list(info.tuned_sweep_ms), "flow_rpl": list(info.flow_rpl), "flow_top": list(info.flow_top),
               "launches_initialize": info.initialize_launches,
               "carrier_sweep_ms": ctx.time_solve(0, reps=5),
               "poisson_sweep_ms": ctx.time_solve(1, reps=5)}
        if args.steady:
            ctx.initialize()
            steps, rel = ctx.run_to_steady_state(MAX_STEPS, TOL, CHECK_EVERY)
            out["steady_steps"] = sorted(int(v) for v in steps)
        print(json.dumps(out))
        return 0
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")

    def one_point():
        ctx.initialize()
        steps, rel = ctx.run_to_steady_state(MAX_STEPS, TOL, CHECK_EVERY)
        return steps, ctx.last_run_steps()

    for _ in range(args.warmup):
        one_point()
    # ---- timed region (device-resident inputs) ------------------------------------
    steps_seen, executed = [], 0
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        ms = 0.0
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0.record(stream)
            s, ex = one_point()
            e1.record(stream)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
            steps_seen.append(int(np.max(s)))
            executed += ex
        torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(ms, world)
    points = args.n_inst * world * args.steps
    value = points / (ms * 1e-3)
    clocks = clk.summary()
    # ---- end-to-end through the public API (host buffers, pinned) --------------------
    ctx.initialize()
    init = {}
    keep = []
    h2d = 0
    for f in range(5):
        if info.ndofs[f]:
            t = torch.empty(args.n_inst * info.ndofs[f], dtype=torch.float64, pin_memory=True)
            a = t.numpy()
            for i in range(args.n_inst):
                a[i * info.ndofs[f]:(i + 1) * info.ndofs[f]] = ctx.get_state(f, i)
            keep.append(t)
            init[f] = a
            h2d += a.nbytes
    d2h = args.n_inst * 8 + sum(args.n_inst * info.ndofs[f] * 8 for f in range(5))
    ctx.iv_sweep(MAX_STEPS, TOL, CHECK_EVERY, init=init, want_fields=True)  # warm
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cur, st_e2e, fin = ctx.iv_sweep(MAX_STEPS, TOL, CHECK_EVERY, init=init, want_fields=True)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = points / e2e_s
    # ---- roofline of the dominant kernel: the carrier solve sweep ---------------------
    ctx.initialize()
    solve_ms = ctx.time_solve(0, reps=30)
    nlaunch = info.solve_launches[0]
    bytes_per_launch = info.solve_bytes[0] / nlaunch
    achieved = bytes_per_launch / (solve_ms * 1e-3 / nlaunch) / 1e9
    peak, peak_kind = load_peaks()
    pois_ms = ctx.time_solve(1, reps=30)
    launches = executed * info.launches_per_step + args.steps * (1 + info.solve_launches[1])
    steps_to_ss = int(statistics.median(steps_seen))
    line = {
        "metric": "I-V points/sec to steady state", "value": value, "unit": "I-V points/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp32ir": "f32 factors + f64 refinement",
                  "mixed": ("f32 factors/quadrature, double-float residuals, increment solves"
                            if args.increment else
                            "f32 factors/quadrature + double-float refinement")}[args.precision],
        "data": "synthetic",
        "config": {"workload": f"half cell 2x{2**args.refine}x{2**args.refine}, LDG k=1, "
                               f"RT0xDGQ0 Poisson, dt=1e-3, to rel. change <= {TOL} "
                               f"(<= {MAX_STEPS} steps)",
                   "instances_per_gpu": args.n_inst, "precision": args.precision,
                   "steps_to_steady_state": steps_to_ss,
                   "l2": "flushed (512 MB write) before each timed I-V point; factors "
                         f"{info.factor_bytes / 1e6:.0f} MB > 129 MB L2"},
        "e2e": {"value": e2e, "unit": "I-V points/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": load_traffic(f"carrier_solve_ref{args.refine}_{args.precision}"),
                     "kernel": "k_forward/k_backward (carrier multifrontal solve sweep)",
                     "solve_ms": solve_ms, "poisson_solve_ms": pois_ms,
                     "bytes_per_sweep": info.solve_bytes[0], "launches_per_sweep": nlaunch},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, steps_to_ss, args.cpu_sample_steps)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def plain_point(pg, refine, local):
    """The plain FP64 single-instance path (half cell 64x64+64x64, k=1): one I-V point."""
    ctx = pg.Context([pg.half_cell(n_refine=refine)], precision=pg.PREC_FP64, device=local)
    ctx.initialize()
    ctx.run_to_steady_state(MAX_STEPS, TOL, CHECK_EVERY)   # warm
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.initialize()
    steps, _ = ctx.run_to_steady_state(MAX_STEPS, TOL, CHECK_EVERY)
    e1.record(stream)
    e1.synchronize()
    return 1.0 / (e0.elapsed_time(e1) * 1e-3), int(steps[0]), ctx


def _fields_of(ctx, i):
    return {f: ctx.get_state(f, i) for f in ctx.fields()}


def _max_rel(a_list, b_list):
    """max over points and fields of ||a - b|| / ||b||"""
    import numpy as np
    worst = 0.0
    for a, b in zip(a_list, b_list):
        for f in b:
            worst = max(worst, float(np.linalg.norm(a[f] - b[f]) / np.linalg.norm(b[f])))
    return worst


def accuracy_block(pg, L, base, thetas, fin, cur, ndofs, local, op, mixed_ctx):
    """The learned + batched answers of `thetas` (fields fin, currents cur)
    against FP64 answers of the same points:
      (i)  the plain method: FP64 from the standard initial condition, stopped
           by the same relative-change rule;
      (ii) the FP64 fixed point: (i) continued to relative change <= 1e-12;
      (iii) precision only: the same warm starts marched in FP64.
    Each is the max over points and fields of the relative L2 error, and the
    max relative error of the interface current."""
    import numpy as np
    n = len(thetas)
    params = [L.instance_params(t, base) for t in thetas]
    ref = pg.Context(params, precision=pg.PREC_FP64, device=local)
    learned = [{f: fin[f][k * ndofs[f]:(k + 1) * ndofs[f]] for f in fin} for k in range(n)]
    ref.initialize()
    s1, _ = ref.run_to_steady_state(MAX_STEPS, TOL, CHECK_EVERY)
    plain = [_fields_of(ref, k) for k in range(n)]
    I1 = ref.interface_current()
    s2, rel2 = ref.run_to_steady_state(2 * MAX_STEPS, 1e-12, CHECK_EVERY)
    fixed = [_fields_of(ref, k) for k in range(n)]
    I2 = ref.interface_current()
    # (iii) the same warm starts in FP64
    init_n, init_p, _, keep = L.warm_start_vectors(mixed_ctx, op, thetas, base)
    s3, I3, fin3 = ref.sweep_stream(params, MAX_STEPS, TOL, CHECK_EVERY, init_n=init_n, init_p=init_p,
                                    want_fields=True)
    del keep
    same = [{f: fin3[f][k * ndofs[f]:(k + 1) * ndofs[f]] for f in fin3} for k in range(n)]
    cur = np.asarray(cur)
    rel = lambda a, b: float(np.max(np.abs(a - b) / np.abs(b)))   # noqa: E731
    out = {
        "points": n,
        "vs_plain_fp64": {"fields_rel_l2_max": _max_rel(learned, plain), "current_rel_max": rel(cur, I1),
                          "reference": "FP64 from the standard initial condition, same stop rule "
                                       f"(rel. change <= {TOL})"},
        "vs_fp64_fixed_point": {"fields_rel_l2_max": _max_rel(learned, fixed), "current_rel_max": rel(cur, I2),
                                "reference": "FP64 marched on to rel. change <= 1e-12",
                                "max_rel_change_reached": float(np.max(rel2))},
        "plain_fp64_vs_fixed_point": {"fields_rel_l2_max": _max_rel(plain, fixed),
                                      "current_rel_max": rel(I1, I2)},
        "precision_only": {"fields_rel_l2_max": _max_rel(learned, same), "current_rel_max": rel(cur, I3),
                           "reference": "the same warm starts marched in FP64"},
        "plain_steps_median": float(np.median(s1)),
    }
    del ref
    return out


def run_full(args):
    """Learned + batched: held-out I-V points streamed through args.batch_inst
    slots (FP32-mixed), each warm-started by the neural operator with the
    first-step fallback, each slot refilled as soon as its point finishes; the
    plain FP64 single-instance path measured beside."""
    import numpy as np
    import torch

    import pecs_gb300 as pg
    from pecs_gb300 import learned as L

    world, rank, local = dist_init(args)
    pg.build()
    B = args.batch_inst
    base = pg.half_cell(n_refine=args.refine)
    # held-out draws (seed differs from the training seed), sharded by rank:
    # warm-up points, timed points, end-to-end points
    n_w, n_t, n_e = args.warmup * B, args.steps * B, args.e2e_waves * B
    per_rank = n_w + n_t + n_e
    thetas = L.sample(per_rank * world, seed=777)[rank * per_rank:(rank + 1) * per_rank]
    th_w, th_t, th_e = thetas[:n_w], thetas[n_w:n_w + n_t], thetas[n_w + n_t:]
    ctx = pg.Context([L.instance_params(t, base) for t in thetas[:B]], precision=pg.PREC_FP32_MIXED,
                     device=local, leaf_cells=args.leaf_cells, flow_sweep=args.flow,
                     increment_solves=bool(args.increment))
    info = ctx.info()
    trained_here = None
    if os.path.exists(args.model):
        op = L.NeuralOperator.load(args.model)
    else:   # no committed model: train a small one now (untimed setup)
        tr = L.sample(args.train_samples, seed=2026)
        Y, _ = L.steady_states(ctx, tr, base)
        op = L.NeuralOperator(rank=32, hidden=256, seed=0)
        T = op.fit_basis(Y, L.Layout.of(ctx))
        op.train(torch.from_numpy(L.normalize(tr)).cuda(), T, epochs=400, batch=64, lr=2e-3)
        trained_here = args.train_samples
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")
    if n_w:
        L.stream_warm_sweep(ctx, op, th_w, base, MAX_STEPS, TOL, CHECK_EVERY)
    # ---- timed: predictions, fallback probes and the streamed sweep of
    # args.steps x B points (parameters uploaded per slot refill; final fields
    # stay on the device) -------------------------------------------------------
    barrier(world)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        flush.zero_()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        steps_t, fb_t, cur_t, _ = L.stream_warm_sweep(ctx, op, th_t, base, MAX_STEPS, TOL, CHECK_EVERY)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        executed = ctx.last_run_steps()
        torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(ms, world)
    points = n_t * world
    value = points / (ms * 1e-3)
    clocks = clk.summary()
    # ---- e2e: host parameters in, currents and final fields out, through the
    # public API (pecs_sweep_stream): e2e_waves x B points, slots refilled ----------
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    steps_e, fb_e, cur_e, fin_e = L.stream_warm_sweep(ctx, op, th_e, base, MAX_STEPS, TOL, CHECK_EVERY,
                                                      want_fields=True)
    e2e = n_e * world / max_over_ranks(time.perf_counter() - t0, world)
    h2d = n_e * (sum(info.ndofs[f] for f in range(5)) * 8 + info.ndofs[4] * 8)  # per-point constant RHS parts
    d2h = n_e * 8 + sum(a.nbytes for a in fin_e.values())
    # ---- a sample of the timed points, batched and streamed without the warm start
    n_nw = min(n_t, 4 * B)
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    steps_nw, _, _, _ = L.stream_warm_sweep(ctx, None, th_t[:n_nw], base, MAX_STEPS, TOL, CHECK_EVERY)
    e3.record(stream)
    e3.synchronize()
    nw_value = n_nw * world / (max_over_ranks(e2.elapsed_time(e3), world) * 1e-3)
    # ---- accuracy of the first B end-to-end points against FP64 answers ------------
    acc = None
    if not args.no_accuracy:
        fin_b = {f: a[:B * info.ndofs[f]] for f, a in fin_e.items()}
        acc = accuracy_block(pg, L, base, th_e[:B], fin_b, cur_e[:B], list(info.ndofs), local, op, ctx)
    # ---- per-stage split of a time step (the reference's TimerOutput sections) ------
    ctx.initialize()
    stages_batched = ctx.time_stages(20)
    # ---- plain path (half cell 64x64+64x64, FP64, single instance) --------------------
    plain_value, plain_steps, pctx = plain_point(pg, args.refine, local)
    pinfo = pctx.info()
    plain_ms = pctx.time_solve(0, reps=30)
    plain_gbs = pinfo.solve_bytes[0] / (plain_ms * 1e-3) / 1e9
    pctx.initialize()
    stages_plain = pctx.time_stages(20)
    del pctx
    # ---- roofline: the carrier solve sweep of the batched path (panel kernels) --------
    solve_ms = ctx.time_solve(0, reps=30)
    nlaunch = info.solve_launches[0]
    achieved = info.solve_bytes[0] / (solve_ms * 1e-3) / 1e9
    peak, peak_kind = load_peaks()
    line = {
        "metric": "I-V points/sec to steady state", "value": value, "unit": "I-V points/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("f32 factors/sweeps, double-float residuals and mass/drift terms, increment solves "
                  if args.increment else
                  "f32 factors/sweeps + double-float refinement ") + "(learned+batched); f64 plain",
        "data": "synthetic",
        "config": {"workload": f"learned+batched: held-out I-V points streamed through {B} slots on the half "
                               f"cell 2x{2**args.refine}x{2**args.refine}, LDG k=1, RT0xDGQ0 Poisson, dt=1e-3, "
                               f"warm-started, to rel. change <= {TOL} (<= {MAX_STEPS} steps)",
                   "bench_step": f"{B} I-V points", "points_timed": n_t, "slots": B,
                   "model": os.path.basename(args.model) if trained_here is None
                   else f"trained in-run on {trained_here} draws",
                   "l2": "flushed (512 MB write) before the timed sweep; the sweep streams ~"
                         f"{info.factor_bytes / 1e6:.0f} MB of factors per step"},
        "plain": {"value": plain_value, "unit": "I-V points/s", "steps_to_steady_state": plain_steps,
                  "workload": "half cell 64x64+64x64, k=1: one instance, FP64 (+1 FP64 refinement sweep per "
                              "solve), standard initial condition"},
        "speedup_vs_plain": value / plain_value,
        "batched_without_warm_start": {"value": nw_value, "unit": "I-V points/s", "points": n_nw,
                                       "median_steps": float(np.median(steps_nw)),
                                       "mean_steps": float(np.mean(steps_nw)),
                                       "capped": int(np.sum(steps_nw >= MAX_STEPS))},
        "warm_start": {"median_steps": float(np.median(steps_t)), "mean_steps": float(np.mean(steps_t)),
                       "capped": int(np.sum(steps_t >= MAX_STEPS + 2)),
                       "fallback_rate": float(np.mean(fb_t)), "plain_steps": plain_steps,
                       "executed_steps": executed},
        "accuracy_vs_fp64": acc,
        "stage_ms_per_step": {"batched_mixed": stages_batched, "plain_fp64": stages_plain,
                              "sections": "carrier RHS, carrier solves, Poisson RHS, Poisson solve "
                                          "(SolarCell.cpp:2057-2075 TimerOutput sections); CUDA events"},
        "e2e": {"value": e2e, "unit": "I-V points/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "points": n_e},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": load_traffic(f"carrier_solve_ref{args.refine}_mixed_b{B}"),
                     "kernel": ("k_panel_flow (carrier multifrontal solve sweep, one persistent "
                                "launch per direction, FP32, " if info.flow_rpl[0] else
                                "k_panel / k_panel_warp (carrier multifrontal solve sweep, one launch "
                                "per tree level, FP32, ") + f"{2 * B} right-hand sides per factor)",
                     "flow_rpl": info.flow_rpl[0], "flow_top": info.flow_top[0],
                     "solve_ms": solve_ms, "launches_per_sweep": nlaunch,
                     "bytes_per_sweep": info.solve_bytes[0],
                     "plain_fp64": {"solve_ms": plain_ms, "achieved_gbs": plain_gbs,
                                    "frac": plain_gbs / peak,
                                    "traffic": load_traffic(f"carrier_solve_ref{args.refine}_fp64")}},
        "gpu_launches": executed * info.launches_per_step,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(args, plain_steps)
        line["cpu_baseline"] = cb
        line["plain_fp64_vs_cpu_baseline"] = plain_value / cb["value"]
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
