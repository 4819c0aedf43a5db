#!/usr/bin/env python
"""Benchmark of the NaSt2D timestep on GB300.

Workload (the plain-method-at-scale configuration): a 4096 x 1024 channel
(dx = dy = 0.01), 64 seeded no-slip rectangles with sides in 4..32, Re = 400,
adaptive step tau = 0.5, gamma = 0.9, omega = 1.7, eps = 1e-3,
max_iterations = 2000, u = 1 on fluid cells at t = 0.  One "step" is one full
run_simulation_tick: boundary pass, F/G, RHS, pressure solve with the
reference's stop rule, velocity update.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` is whole-job cell-updates/s (interior cells x
steps / device time) of the plain FP64 red-black path, inputs resident in
HBM; `e2e` is the same metric through the public API with host (pinned)
buffers uploaded and downloaded every step.  Under torchrun each rank runs
its own replica (weak scaling).  Further blocks on rank 0:

* `mixed_precision`: FP32 sweeps + FP64 norm/refinement on the same
  workload (autotuned sweep schedule), its speed-up over the plain path and
  each field's error against the plain FP64 run after `--err-steps` steps;
* `learned`: the BF16 U-Net warm start, trained here on snapshots of
  512 x 128 channels, judged in the loop on the same workload against the
  mixed solve from identical states (sweeps to the same residual, time);
* `cavity_mixed`: the 2048 x 2048 lid-driven cavity (Re 1000, omega 1.8,
  eps 1e-5 on the residual relative to the solve's start), mixed against
  FP64: Poisson time-to-residual per step and the fields' error;
* `batched`: many channel simulations of uneven sizes stepped as one batch
  against the same instances run one after another on the plain FP64 path.

`--impl reference` times the reference algorithm's CPU restatement (the
oracle; the Rust crate cannot be built here) on bounded samples of the same
workload.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

IMAX, JMAX = 4096, 1024
NRECTS, SEED = 64, 0
PARAMS = dict(cell_size=(0.01, 0.01), delt=0.005, gamma=0.9, reynolds=400.0,
              sor_absolute_epsilon=1e-3, max_iterations=2000, omega=1.7, tau=0.5)
# delt is the adaptive rule's value at t = 0 (u = 1): 0.5 * min(Re/2/(2/dx^2), dx/1)
CELLS = IMAX * JMAX
# iterations per WHILE body of the FAST solve's step graph (the library's
# kFastBodyIters)
FAST_BODY_ITERS = 8
L2_BYTES = 129e6
# the warm-start network's parameters, trained at 512 x 128 outside the
# benchmark (python -m stroemung_gb300.train_warmstart)
WS_WEIGHTS = ROOT / "stroemung_gb300" / "weights" / "warmstart_unet_channel_512x128.npy"


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def load_bf16_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("bf16_tflops", 1900.0))
    return 1900.0


BF16_PEAK = load_bf16_peak()


def workload(seed: int):
    from stroemung_gb300 import presets
    rects = presets.random_rectangles(IMAX, JMAX, NRECTS, seed)
    return presets.channel(IMAX, JMAX, rects)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "samples": len(sm), "reasons": sorted(reasons)}


def oracle_sim(grid, red_black: bool = False, threads: int = 1):
    """The oracle (the reference's algorithm restated in C: lexicographic SOR
    in its x-major order, FP64, one thread) on `grid` with the workload's
    parameters; red_black / threads select the oracle's red-black order with
    its sweeps and norm on several threads (a multi-core CPU for comparison,
    not the reference's own code path)."""
    from oracle import oracle as orc
    orc.build()
    p = PARAMS
    o = orc.OracleSim(kind=grid["kind"], wall_uv=grid["wall_uv"], u=grid["u"], v=grid["v"],
                      p=grid["p"], dx=p["cell_size"][0], dy=p["cell_size"][1],
                      delt=p["delt"], gamma=p["gamma"], reynolds=p["reynolds"],
                      eps=p["sor_absolute_epsilon"], omega=p["omega"],
                      max_iterations=p["max_iterations"], tau=p["tau"],
                      sor_order=orc.RED_BLACK if red_black else orc.LEXICOGRAPHIC)
    if threads > 1:
        o.set_threads(threads)
    return o


def cpu_phases(grid, ticks: int, cap: int, red_black: bool = False, threads: int = 1):
    """Times `ticks` oracle ticks of the full workload with the solve capped
    at `cap` iterations: mean seconds before the solve, per solve iteration
    and after it, and the wall time."""
    o = oracle_sim(grid, red_black, threads)
    pre, it_s, post = [], [], []
    t0 = time.perf_counter()
    for _ in range(ticks):
        a, b, n, c = o.tick_timed(cap)
        pre.append(a)
        post.append(c)
        if n > 0:
            it_s.append(b / n)
    wall = time.perf_counter() - t0
    return (statistics.mean(pre), statistics.mean(it_s) if it_s else 0.0,
            statistics.mean(post), wall)


def cpu_sample(grid, k_iters: float, ticks: int, cap: int):
    """The oracle's step time for a step of k_iters iterations, from `ticks`
    capped ticks (phase times measured, iterations scaled)."""
    pre, t_iter, post, wall = cpu_phases(grid, ticks, cap)
    return pre + k_iters * t_iter + post, t_iter, wall


def run_reference(args):
    """The reference arm: the oracle on the host, one thread (the reference's
    ndarray loops are single-threaded), on the same workload.  Each of the
    warmup + steps samples is one tick with the solve capped at --ref-cap
    iterations, its step time modelled as pre-solve + max_iterations x the
    per-iteration time + post-solve (every step this workload's GPU arm times
    runs max_iterations); then the first 1 + --ref-full-steps uncapped ticks
    from the workload's start are timed whole, and the model's error against
    the ticks after the first (which run max_iterations) is reported."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    grid = workload(SEED)
    k = PARAMS["max_iterations"]
    phases = []
    for i in range(args.warmup + args.steps):
        ph = cpu_phases(grid, 1, args.ref_cap)
        if i >= args.warmup:
            phases.append(ph)
    pre = statistics.mean(x[0] for x in phases)
    t_iter = statistics.mean(x[1] for x in phases)
    post = statistics.mean(x[2] for x in phases)
    t = pre + k * t_iter + post
    value = CELLS / t
    sample = (f"each step: one oracle tick of the full 4096x1024 workload with the pressure "
              f"solve capped at {args.ref_cap} iterations; step time = measured pre-solve + "
              f"{k} x measured per-iteration + measured post-solve time ({k} = "
              f"max_iterations, what this configuration's solve runs per step)")
    full = None
    if args.ref_full_steps > 0:
        # whole ticks from the workload's start: the first tick's solve stops
        # after a few iterations (its norm drops below the initial norm at
        # once); from the second on every tick runs max_iterations, as in the
        # window the GPU arm times, so the model is checked on those
        o = oracle_sim(grid)
        ticks = []
        for i in range(1 + args.ref_full_steps):
            t0 = time.perf_counter()
            it, ns = o.tick()
            ticks.append((it, time.perf_counter() - t0))
            print(f"reference tick {i + 1}: {it} iterations, norm {ns:.6e}, "
                  f"{ticks[-1][1]:.2f} s", file=sys.stderr, flush=True)
        # the model is checked on the ticks it is quoted for: those after the
        # first that run max_iterations (all of them when none does)
        sel = [(it, w) for it, w in ticks[1:] if it == k] or ticks[1:]
        measured = statistics.mean(w for _, w in sel)
        model = pre + statistics.mean(it for it, _ in sel) * t_iter + post
        total = sum(w for _, w in ticks)
        total_model = sum(pre + it * t_iter + post for it, _ in ticks)
        full = {"ticks": [{"sor_iterations": it, "ms": w * 1e3} for it, w in ticks],
                "measured_full_step_ms": measured * 1e3, "model_full_step_ms": model * 1e3,
                "model_error": (model - measured) / measured,
                "measured_value": CELLS / measured,
                "whole_run_s": total, "whole_run_model_s": total_model,
                "whole_run_sweeps": sum(it for it, _ in ticks),
                "whole_run_value": CELLS * len(ticks) / total,
                "bound": "the model is accepted when |model_error| <= 0.05",
                "note": "uncapped oracle ticks from the workload's start, timed whole; "
                        "measured_full_step_ms averages the ticks after the first that run "
                        f"{k} iterations; the model is the sampled steps' pre-solve + "
                        "iterations x per-iteration + post-solve time for the same iteration "
                        "counts; whole_run_* cover every tick"}
    # beside it, labelled: the same algorithm on every host core (the
    # oracle's red-black order, its sweeps and norm threaded; the rest of
    # the tick serial) — what a multi-core CPU does, not the reference's code
    parallel = None
    nthreads = os.cpu_count() or 1
    if args.ref_parallel and nthreads > 1:
        ph = [cpu_phases(grid, 1, args.ref_cap, red_black=True, threads=nthreads)
              for _ in range(2)]
        pt = (statistics.mean(x[0] for x in ph) + k * statistics.mean(x[1] for x in ph) +
              statistics.mean(x[2] for x in ph))
        parallel = {"value": CELLS / pt, "unit": "cell-updates/s", "ms_per_step": pt * 1e3,
                    "threads": nthreads,
                    "sample": f"2 oracle ticks, red-black order, the SOR sweeps and the norm on "
                              f"{nthreads} threads (the rest of the tick on one), solve capped "
                              f"at {args.ref_cap} iterations; step time = pre-solve + {k} x "
                              f"per-iteration + post-solve"}
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(args, reference=True),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                         "sample": sample, "host_cpu": os.uname().machine,
                         "nproc": os.cpu_count()},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if full is not None:
        line["full_step"] = full
    if parallel is not None:
        line["cpu_all_cores_red_black"] = parallel
    print(json.dumps(line))


METRIC = "cell-updates/s (4096x1024 channel timestep, FP64 red-black SOR)"

# DRAM traffic from the committed ncu captures of this workload (bytes):
# one FP64 iteration (red pass 73.2 + 0.9 MB, black pass 72.5 + 0.2 MB: the
# updated pressures stay in L2, written back later) and one FP32 sweep (a
# 4-sweep blocked launch: 38.4 + 49.9 MB).
SOR_ITERATION_TRAFFIC = (73.2 + 0.9 + 72.5 + 0.2) * 1e6
SWEEP_TRAFFIC = (38.4 + 49.9) * 1e6 / 4


def config_dict(args, reference: bool = False):
    solver = ("lexicographic SOR (x outer, y inner), FP64, the reference's operation order, "
              "one thread" if reference else f"red-black SOR, FP64, {args.arith} arithmetic")
    return {"workload": "channel 4096x1024, 64 rectangles (seed 0), Re 400, tau 0.5, "
                        "eps 1e-3, max_iterations 2000",
            "imax": IMAX, "jmax": JMAX, "obstacles": NRECTS,
            "solver": solver,
            "stop_rule": "reference (ns < initial norm or ns < eps^2)",
            "l2": "per-step working set (9 FP64 fields + flags, 285 MB) exceeds the 129 MB L2; "
                  "no flush", "parallelism": f"replicas x{args.gpus}"}


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest rank's time (replicas run independently; the whole job
    ends with the last one)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(cells_per_step: float, steps: int, world: int, seconds: float) -> float:
    """Whole-job cell-updates/s of `world` replicas, each doing `steps`
    steps of `cells_per_step`, the job taking `seconds` (max over ranks)."""
    return cells_per_step * steps * world / seconds


def field_errors(a_fields, b_fields, fluid):
    """Relative L2 and max abs error per field; the pressure on fluid cells
    with its mean removed (pure Neumann: each solve fixes its own constant)."""
    import numpy as np
    err = {}
    for n in ("u", "v", "p"):
        a, b = a_fields[n], b_fields[n]
        if n == "p":
            a, b = a[fluid] - a[fluid].mean(), b[fluid] - b[fluid].mean()
        err[n] = {"rel_l2": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)),
                  "max_abs": float(np.abs(a - b).max())}
    return err


def timed_steps(sim, n, stream):
    import torch
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stats = sim.step_n(n)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), stats


def error_growth(args, grid):
    """Field errors against the plain FP64 (fast arithmetic) run, stepped in
    lockstep from the same initial state: the mixed-precision solve, and as a
    control the FP64 run with the reference's exact operation order (the
    two FP64 runs differ only by rounding)."""
    from stroemung_gb300.simulation import PREC_MIXED, ARITH_EXACT, ARITH_FAST, Simulation
    fast = Simulation(grid=grid, arithmetic=ARITH_FAST, **PARAMS)
    exact = Simulation(grid=grid, arithmetic=ARITH_EXACT, **PARAMS)
    mixed = Simulation(grid=grid, precision=PREC_MIXED, inner_sweeps=args.inner_sweeps,
                       arithmetic=ARITH_FAST, **PARAMS)
    fluid = grid["kind"] == 0
    checkpoints = sorted({c for c in (1, 5, 10, 25, 50, args.err_steps) if c <= args.err_steps})
    rows = []
    done = 0
    iters = {"fast": [], "exact": [], "mixed": []}
    for c in checkpoints:
        for name, sim in (("fast", fast), ("exact", exact), ("mixed", mixed)):
            iters[name] += [s[0] for s in sim.step_n(c - done)]
        done = c
        ref = {n: fast.download(n) for n in ("u", "v", "p")}
        em = field_errors({n: mixed.download(n) for n in ("u", "v", "p")}, ref, fluid)
        ex = field_errors({n: exact.download(n) for n in ("u", "v", "p")}, ref, fluid)
        rows.append({"step": c, "mixed": {k: v["rel_l2"] for k, v in em.items()},
                     "fp64_exact_order": {k: v["rel_l2"] for k, v in ex.items()}})
    for sim in (fast, exact, mixed):
        sim.close()
    # steps whose pressure solve stopped after a different number of sweeps
    # than the FP64 run's (step number, FP64 sweeps, other run's sweeps)
    differ = {n: [(i + 1, a, b) for i, (a, b) in enumerate(zip(iters["fast"], iters[n])) if a != b]
              for n in ("mixed", "exact")}
    return {"rel_l2_by_step": rows, "sweep_count_differs": differ}


def mixed_block(args, grid, fp64_ms_step, peak):
    """Mixed precision on the same workload, from the same initial state."""
    import torch
    from stroemung_gb300.simulation import PREC_MIXED, ARITH_FAST, Simulation
    sim = Simulation(grid=grid, precision=PREC_MIXED, inner_sweeps=args.inner_sweeps,
                     arithmetic=ARITH_FAST, **PARAMS)
    stream = torch.cuda.ExternalStream(sim.device_view()["stream"])
    warm = sim.step_n(args.warmup)
    best, sched_ms = sim.autotune_sweeps(reps=3)
    ms, stats = timed_steps(sim, args.steps, stream)
    iters = [x[0] for x in stats]
    # the FP32 sweeps alone (the dominant kernel of this path), timed live
    nsw = 16 * 4
    sw0 = torch.cuda.Event(enable_timing=True)
    sw1 = torch.cuda.Event(enable_timing=True)
    sim.synchronize()
    sw0.record(stream)
    sim.sor_sweeps(nsw, wait=False)
    sw1.record(stream)
    sim.synchronize()
    t_sw = sw0.elapsed_time(sw1) / 1e3 / nsw
    sw_bytes = 13.0 * CELLS  # read e, s (8) + flags (1), write e (4)
    sim.close()
    # the step time at other refinement intervals (same stop sweeps: the loop
    # redoes the last interval sweep by sweep when the rule fires inside it)
    by_inner = {}
    for m in args.inner_alt:
        alt = Simulation(grid=grid, precision=PREC_MIXED, inner_sweeps=m, arithmetic=ARITH_FAST,
                         **PARAMS)
        alt.step_n(1)
        alt.autotune_sweeps(reps=2)
        st_alt = torch.cuda.ExternalStream(alt.device_view()["stream"])
        ms_alt, _ = timed_steps(alt, 3, st_alt)
        by_inner[str(m)] = {"ms_per_step": ms_alt / 3,
                            "speedup_vs_fp64": fp64_ms_step / (ms_alt / 3)}
        alt.close()
    growth = error_growth(args, grid) if args.err_steps > 0 else {"rel_l2_by_step": [],
                                                                  "sweep_count_differs": {}}
    return {
        "value": CELLS * args.steps / (ms / 1e3), "unit": "cell-updates/s",
        "ms_per_step": ms / args.steps, "speedup_vs_fp64": fp64_ms_step / (ms / args.steps),
        "inner_sweeps": min(args.inner_sweeps, PARAMS["max_iterations"]),
        "other_inner_sweeps": by_inner,
        "sweep_schedule": {"chosen": best, "us_per_sweep": {str(k): v * 1e3
                                                            for k, v in sched_ms.items()},
                           "note": "1 = one launch per colour pass; 2..7 = shared-memory "
                                   "tiles with 2-8 sweeps per launch (autotuned here)"},
        "sor_iterations": {"mean": statistics.mean(iters), "min": min(iters), "max": max(iters),
                           "warmup": [w[0] for w in warm]},
        "error_vs_fp64": {
            **growth,
            "note": "relative L2 against the plain FP64 run (pressure on fluid cells, mean "
                    "removed); the FP64 exact-order run is the control: it differs from the "
                    "plain run by rounding only, and both errors grow at the flow's rate"},
        "roofline_fp32_sweep": {"achieved": sw_bytes / t_sw / 1e9, "peak": peak, "unit": "GB/s",
                                "frac": sw_bytes / t_sw / 1e9 / peak, "us_per_sweep": t_sw * 1e6,
                                "algorithmic_bytes": sw_bytes,
                                "traffic": SWEEP_TRAFFIC,
                                "traffic_note": "ncu dram__bytes read+write of one blocked "
                                                "launch (4 sweeps) of this workload divided "
                                                "by 4, cold cache: the sweeps read e, s and "
                                                "the flags once per launch"},
        "dtype": "f32 stencil and sweeps, f64 norm/refinement/dt",
    }


def run_lengths(xs):
    """[[count, value], ...] of consecutive equal values."""
    out = []
    for x in xs:
        if out and out[-1][1] == x:
            out[-1][0] += 1
        else:
            out.append([1, x])
    return out


def full_run_block(args, grid):
    """The whole configuration: --full-steps steps (500) of the workload from
    its start, in FP64 (fast arithmetic) and in mixed precision.  Each step is
    issued as its two graph halves (boundary pass, F/G, RHS; pressure solve,
    velocity update) with CUDA events around each, so the time of both
    phases is measured per step."""
    import torch
    from stroemung_gb300.simulation import ARITH_FAST, PREC_FP64, PREC_MIXED, Simulation
    out = {}
    n = args.full_steps
    for label, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        kw = dict(grid=grid, arithmetic=ARITH_FAST, precision=prec,
                  inner_sweeps=args.inner_sweeps, **PARAMS)
        sched = 0
        if prec == PREC_MIXED:
            tmp = Simulation(**kw)
            tmp.step_n(1)
            sched, _ = tmp.autotune_sweeps(reps=2)
            tmp.close()
        sim = Simulation(sweep_schedule=sched, **kw)
        stream = torch.cuda.ExternalStream(sim.device_view()["stream"])
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(n)]
        iters = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(n):
            ev[k][0].record(stream)
            sim.tick_prepare()
            ev[k][1].record(stream)
            it, _ = sim.tick_solve()
            ev[k][2].record(stream)
            iters.append(it)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        prep = [ev[k][0].elapsed_time(ev[k][1]) for k in range(n)]
        solve = [ev[k][1].elapsed_time(ev[k][2]) for k in range(n)]
        dev_s = (sum(prep) + sum(solve)) / 1e3
        itermax = PARAMS["max_iterations"]
        full = [k for k, it in enumerate(iters) if it >= itermax]
        short = [it for it in iters if it < itermax]
        out[label] = {
            "steps": n, "device_s": dev_s, "wall_s": wall,
            "value": CELLS * n / dev_s, "unit": "cell-updates/s",
            "prepare_ms_total": sum(prep), "solve_ms_total": sum(solve),
            "prepare_ms_per_step": sum(prep) / n,
            "solve_ms_per_step_at_itermax": statistics.mean(solve[k] for k in full) if full
            else None,
            "solve_ms_per_step_below_itermax": statistics.mean(
                solve[k] for k in range(n) if iters[k] < itermax) if short else None,
            "sweeps_total": sum(iters), "steps_at_itermax": len(full),
            "last_step_at_itermax": (full[-1] + 1) if full else None,
            "mean_sweeps_below_itermax": statistics.mean(short) if short else None,
            "sweeps_per_step": run_lengths(iters)}
        if prec == PREC_MIXED:
            out[label]["sweep_schedule"] = sched
        sim.close()
    out["mixed_speedup_vs_fp64"] = out["fp64"]["device_s"] / out["mixed"]["device_s"]
    out["note"] = ("device_s sums the two halves' CUDA-event times of every step; wall_s "
                   "includes the host's per-step read of the iteration count")
    return out


def learned_block(args, grid, fp64_ms_step, mixed_ms_step):
    """Train the U-Net on 512 x 128 snapshots, then step the workload with the
    judged warm start, each step A/B against the plain mixed solve from the
    identical state."""
    import numpy as np
    import torch
    from stroemung_gb300 import warmstart
    from stroemung_gb300.simulation import PREC_MIXED, ARITH_FAST, Simulation
    from stroemung_gb300.unet import UNet
    from stroemung_gb300.train_warmstart import load_weights
    net = UNet(seed=0)
    train_info = {}
    weights = args.ws_weights or (str(WS_WEIGHTS) if WS_WEIGHTS.exists() else "")
    if weights:
        sha = load_weights(net, weights)
        train_info = {"weights": os.path.basename(weights), "weights_sha256": sha,
                      "note": "trained outside the benchmark by stroemung_gb300.train_warmstart "
                              "(512 x 128 channel snapshots, Adam, batch 32, error loss)"}
    else:
        t0 = time.perf_counter()
        train = warmstart.generate_snapshots(args.ws_snapshots, imax=512, jmax=128,
                                             steps_per_problem=32, seed=11)
        held = warmstart.generate_snapshots(64, imax=512, jmax=128, steps_per_problem=32,
                                            seed=12)
        t_gen = time.perf_counter() - t0
        tr = warmstart.Trainer(net, 514, 130, 0.01, 0.01, batch=32)
        before, _ = tr.loss(held, 0)
        t0 = time.perf_counter()
        hist = tr.fit(train, epochs=args.ws_epochs, lr=1e-3)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t0
        after, _ = tr.loss(held, 0)
        train_info = {"snapshots": args.ws_snapshots, "grid": "512x128", "epochs": args.ws_epochs,
                      "adam_steps": len(hist), "batch": 32, "lr": 1e-3,
                      "held_out_relative_residual": {"before": before, "after": after},
                      "generate_s": t_gen, "train_s": t_train,
                      "train_ms_per_step": t_train / max(len(hist), 1) * 1e3}
        del train, held, tr
        torch.cuda.empty_cache()
    # forward cost at the workload size and its tensor-pipe rate
    x = torch.zeros(1, IMAX, JMAX, 8, dtype=torch.bfloat16, device="cuda")
    net.forward(x, 1, IMAX, JMAX)
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record()
    for _ in range(3):
        net.forward(x, 1, IMAX, JMAX)
    f1.record()
    torch.cuda.synchronize()
    fwd_ms = f0.elapsed_time(f1) / 3
    # the prediction's forward as the warm start runs it (recorded once as a
    # CUDA graph and replayed: no activation kept for a backward, the last
    # layer's outputs not stored, no host work between the launches)
    net.forward_graphed(x, 1, IMAX, JMAX)
    torch.cuda.synchronize()
    f0.record()
    for _ in range(3):
        net.forward_graphed(x, 1, IMAX, JMAX)
    f1.record()
    torch.cuda.synchronize()
    pred_fwd_ms = f0.elapsed_time(f1) / 3
    flops = 0.0
    pixel_scale = [1, 1, 4, 4, 16, 16, 64, 64, 16, 16, 4, 4, 1, 1]  # pixels per layer: 1/scale
    for l, sc in zip(net.layers(), pixel_scale):
        flops += 2.0 * 9 * l.cin * l.cout * IMAX * JMAX / sc
    del x
    net._bufs.clear()
    torch.cuda.empty_cache()
    mk = dict(precision=PREC_MIXED, inner_sweeps=args.inner_sweeps, arithmetic=ARITH_FAST)
    plain = Simulation(grid=grid, **mk, **PARAMS)
    wsim = Simulation(grid=grid, **mk, **PARAMS)
    ws = warmstart.WarmStartSolver(wsim, net, judge_sweeps=args.ws_judge_sweeps)
    ws.warm_up()
    scratch = torch.zeros(IMAX + 2, JMAX + 2, dtype=torch.float64, device="cuda")
    plain.step_n(args.warmup)
    warmstart.sync_state(wsim, plain, scratch)
    rows = []
    for _ in range(args.ws_steps):
        r = warmstart.compare_step(plain, ws, scratch)
        hp, hw = r.pop("hist_plain"), r.pop("hist_ws")
        # sweeps each run needs to first reach the plain run's norm at 1/8,
        # 1/2 and all of its sweeps (first reach in both: the reference norm
        # is not monotone over a solve)
        marks = {}
        for frac in (0.125, 0.5, 1.0):
            k = max(0, min(len(hp) - 1, int(round(frac * (len(hp) - 1)))))
            target = hp[k, 1]
            marks[str(frac)] = {"plain": warmstart.sweeps_to_reach(hp, target),
                                "learned": warmstart.sweeps_to_reach(hw, target)}
        r["sweeps_to_plain_norm"] = marks
        r["plain_sweeps_to_plain_final"] = warmstart.sweeps_to_reach(hp, hp[-1, 1])
        rows.append(r)
    # the learned step as a user runs it: predict, judge, solve
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.ws_steps):
        ws.step()
    torch.cuda.synchronize()
    learned_ms = (time.perf_counter() - t0) / args.ws_steps * 1e3
    plain.close()
    wsim.close()
    acc = sum(1 for r in rows if r["accepted"])
    ratio = [r["ns_pred"] / r["ns_prev"] for r in rows if r["ns_prev"] > 0]
    # sweeps saved to the plain run's final norm (first reach against first
    # reach) count only where the plain solve lowered its norm: the
    # reference norm (obstacle cells included) can end a solve above where
    # it started, and then any start that is not worse "reaches" it at once
    saved = [r["plain_sweeps_to_plain_final"] - r["ws_sweeps_to_plain_final"] for r in rows
             if r["ws_sweeps_to_plain_final"] is not None and r["ns_plain"] < r["ns0_plain"]]
    rose = sum(1 for r in rows if r["ns_plain"] >= r["ns0_plain"])
    return {
        "value": CELLS / (learned_ms / 1e3), "unit": "cell-updates/s",
        "ms_per_step": learned_ms, "speedup_vs_fp64": fp64_ms_step / learned_ms,
        "speedup_vs_mixed": mixed_ms_step / learned_ms if mixed_ms_step else None,
        "predict_ms": statistics.mean(r["predict_ms"] for r in rows),
        "judge_ms": statistics.mean(r["judge_ms"] for r in rows),
        "accepted": f"{acc}/{len(rows)}",
        "initial_norm_ratio_median": statistics.median(ratio) if ratio else None,
        "sweeps_saved_to_plain_final_norm": {"per_step": saved, "steps_reaching": len(saved),
                                             "steps": len(rows),
                                             "steps_where_plain_norm_rose": rose},
        "final_norm_ratio_at_equal_sweeps": [r["ns_ws"] / r["ns_plain"] for r in rows
                                             if r["ns_plain"] > 0],
        "per_step": [{k: r[k] for k in ("sweeps_plain", "sweeps_ws", "ns0_plain", "ns_plain",
                                         "ns_ws", "ns_prev", "ns_pred", "accepted",
                                         "sweeps_to_plain_norm")} for r in rows],
        "cnn": {"forward_ms_at_workload": fwd_ms, "forward_tflops": flops / fwd_ms / 1e9,
                "tensor_frac_of_measured_bf16": (flops / fwd_ms / 1e9) / BF16_PEAK,
                "prediction_forward_ms": pred_fwd_ms,
                "prediction_tensor_frac_of_measured_bf16": (flops / pred_fwd_ms / 1e9) /
                BF16_PEAK,
                "params": net.parameter_count(),
                "note": "forward_ms_at_workload: forward() keeping every activation for a "
                        "backward, host calls between the launches; prediction_forward_ms: the "
                        "warm start's recorded forward graph, storing no activation it does not "
                        "read"},
        "training": train_info,
        "judge_sweeps": args.ws_judge_sweeps,
        "note": "the reference stop rule runs 2000 sweeps in every step of this workload, so no "
                "warm start can save sweeps here; sweeps_to_plain_norm counts the sweeps each "
                "run needs to reach the plain run's norms; see learned_cavity for a converging "
                "case",
    }


def learned_cavity_block(args):
    """The warm start where solves converge: n x n lid-driven cavities (Re
    log-uniform in [50, 2000], strict eps 1e-3 on the mean-free fluid
    residual).  Two configurations, each trained here on the same snapshots
    and stepped A/B against the plain mixed solve from identical states on
    two held-out Reynolds numbers: the residual loss with the initial-residual
    judge, and the error loss (against the solved pressure) with the judge
    after judge_sweeps red-black iterations."""
    import numpy as np
    import torch
    from stroemung_gb300 import presets, warmstart
    from stroemung_gb300.unet import UNet
    n = args.ws_cavity_n
    fam = warmstart.cavity_family(n)
    t0 = time.perf_counter()
    train = warmstart.generate_snapshots(args.ws_snapshots, family=fam, steps_per_problem=32,
                                         seed=1, targets=True)
    t_gen = time.perf_counter() - t0
    out = {"grid": f"{n}x{n}", "snapshots": args.ws_snapshots, "generate_s": t_gen,
           "stop_rule": "ns < (1e-3)^2, fluid cells, mean removed", "held_out_re": [150.0, 900.0],
           "steps_per_re": args.ws_cavity_steps}
    for name, loss, judge in (("residual_loss_initial_judge", "residual", 0),
                              ("error_loss_smoothed_judge", "error", args.ws_judge_sweeps)):
        net = UNet(seed=0)
        tr = warmstart.Trainer(net, n + 2, n + 2, 1.0 / n, 1.0 / n, batch=32, loss=loss)
        t0 = time.perf_counter()
        hist = tr.fit(train, epochs=args.ws_cavity_epochs, lr=1e-3)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t0
        sp = sw = acc = steps = 0
        t_plain = t_ws = t_pred = t_judge = 0.0
        for re in out["held_out_re"]:
            plain = warmstart.make_simulation(presets.cavity(n), re, 1.0 / n, delt=1e-3,
                                              max_iterations=40000)
            wsim = warmstart.make_simulation(presets.cavity(n), re, 1.0 / n, delt=1e-3,
                                             max_iterations=40000)
            ws = warmstart.WarmStartSolver(wsim, net, judge_sweeps=judge)
            ws.warm_up()
            scratch = torch.zeros(n + 2, n + 2, dtype=torch.float64, device="cuda")
            for _ in range(args.ws_cavity_steps):
                r = warmstart.compare_step(plain, ws, scratch)
                sp += r["sweeps_plain"]
                sw += r["sweeps_ws"]
                acc += r["accepted"]
                steps += 1
                t_plain += r["solve_plain_ms"]
                t_ws += r["predict_ms"] + r["judge_ms"] + r["solve_ws_ms"]
                t_pred += r["predict_ms"]
                t_judge += r["judge_ms"]
            plain.close()
            wsim.close()
        out[name] = {"loss": loss, "judge_sweeps": judge, "epochs": args.ws_cavity_epochs,
                     "train_s": t_train, "loss_first_last": [float(np.mean(hist[:8])),
                                                             float(np.mean(hist[-8:]))],
                     "sweeps_plain": sp, "sweeps_learned": sw, "sweeps_saved": 1 - sw / sp,
                     "accepted": f"{acc}/{steps}", "ms_plain": t_plain,
                     "ms_learned_incl_predict_and_judge": t_ws,
                     "predict_ms_per_step": t_pred / steps, "judge_ms_per_step": t_judge / steps,
                     "time_saved": 1 - t_ws / t_plain}
    return out


def cavity_block(args):
    """Lid-driven cavity 2048 x 2048, Re 1000, omega 1.8, eps 1e-5 relative:
    FP64 and mixed from the same state; Poisson time-to-residual per step."""
    import numpy as np
    import torch
    from stroemung_gb300 import presets
    from stroemung_gb300.simulation import PREC_FP64, PREC_MIXED, ARITH_FAST, Simulation
    n = args.cavity_n
    grid = presets.cavity(n)
    cfg = dict(cell_size=(1.0 / n, 1.0 / n), delt=1e-4, gamma=0.9, reynolds=1000.0,
               sor_absolute_epsilon=1e-5, max_iterations=args.cavity_itermax, omega=1.8,
               tau=0.5, arithmetic=ARITH_FAST, strict_eps=2)
    out = {"grid": f"{n}x{n}", "steps": args.cavity_steps, "max_iterations": args.cavity_itermax,
           "stop_rule": "ns < (1e-5)^2 x the norm the solve starts from"}
    res = {}
    fields = {}
    for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        sim = Simulation(grid=grid, precision=prec, **cfg)
        stream = torch.cuda.ExternalStream(sim.device_view()["stream"])
        per = []
        for _ in range(args.cavity_steps):
            ms, st = timed_steps(sim, 1, stream)
            per.append((ms, int(st[0][0]), bool(st[0][3])))
        fields[name] = {k: sim.download(k) for k in ("u", "v", "p")}
        sim.close()
        res[name] = {"ms_per_step": [p[0] for p in per], "sweeps": [p[1] for p in per],
                     "converged": [p[2] for p in per],
                     "time_to_residual_ms_median": statistics.median(p[0] for p in per)}
    out.update(res)
    out["speedup_mixed_vs_fp64"] = (sum(res["fp64"]["ms_per_step"]) /
                                    sum(res["mixed"]["ms_per_step"]))
    out["error_mixed_vs_fp64"] = field_errors(fields["mixed"], fields["fp64"], grid["kind"] == 0)
    if args.cavity_small:
        out["converging"] = time_to_residual(args.cavity_small, args.cavity_steps)
    return out


def cavity_run(args):
    """The 2048 x 2048 lid-driven cavity (Re 1000, omega 1.8, tau 0.5, eps
    1e-5 on the residual relative to each solve's starting norm) for
    --cavity-run steps, FP64 (fast arithmetic) and mixed precision stepped in
    lockstep from the same state, each solve capped at --cavity-run-itermax
    sweeps.  Per step: device time, sweeps and the relative residual each
    solve reached (from its residual history); every --cavity-run-every steps
    the fields' relative L2 and max error of mixed against FP64.  Prints one
    JSON document (not a benchmark line)."""
    import numpy as np
    import torch
    from stroemung_gb300 import presets
    from stroemung_gb300.simulation import PREC_FP64, PREC_MIXED, ARITH_FAST, Simulation
    n = args.cavity_n
    grid = presets.cavity(n)
    fluid = grid["kind"] == 0
    cfg = dict(grid=grid, cell_size=(1.0 / n, 1.0 / n), delt=1e-4, gamma=0.9,
               reynolds=1000.0, sor_absolute_epsilon=1e-5,
               max_iterations=args.cavity_run_itermax, omega=1.8, tau=0.5,
               arithmetic=ARITH_FAST, strict_eps=2)
    tmp = Simulation(precision=PREC_MIXED, **cfg)
    tmp.step_n(1)
    sched, _ = tmp.autotune_sweeps(reps=2)
    tmp.close()
    sims = {"fp64": Simulation(precision=PREC_FP64, **cfg),
            "mixed": Simulation(precision=PREC_MIXED, sweep_schedule=sched, **cfg)}
    streams = {k: torch.cuda.ExternalStream(v.device_view()["stream"]) for k, v in sims.items()}
    rows = {k: {"ms": [], "sweeps": [], "rel_residual": [], "converged": []} for k in sims}
    errors = []
    for step in range(1, args.cavity_run + 1):
        for k, sim in sims.items():
            ms, st = timed_steps(sim, 1, streams[k])
            h = sim.residual_history()
            rel = float(np.sqrt(h[-1, 1] / h[0, 1])) if len(h) and h[0, 1] > 0 else None
            rows[k]["ms"].append(ms)
            rows[k]["sweeps"].append(int(st[0][0]))
            rows[k]["rel_residual"].append(rel)
            rows[k]["converged"].append(bool(st[0][3]))
        if step % args.cavity_run_every == 0 or step == args.cavity_run:
            f = {k: {n_: sim.download(n_) for n_ in ("u", "v", "p")} for k, sim in sims.items()}
            errors.append({"step": step, **field_errors(f["mixed"], f["fp64"], fluid)})
    for sim in sims.values():
        sim.close()
    out = {"grid": f"{n}x{n}", "steps": args.cavity_run,
           "max_iterations": args.cavity_run_itermax, "sweep_schedule_mixed": sched,
           "stop_rule": "ns < (1e-5)^2 x the norm the solve starts from, capped at "
                        "max_iterations sweeps",
           "errors_mixed_vs_fp64": errors}
    for k, r in rows.items():
        out[k] = {"device_s": sum(r["ms"]) / 1e3,
                  "ms_per_step_median": statistics.median(r["ms"]),
                  "steps_converged": sum(r["converged"]),
                  "sweeps_per_step": run_lengths(r["sweeps"]),
                  "rel_residual_per_step": r["rel_residual"],
                  "ms_per_step": r["ms"]}
    out["speedup_mixed_vs_fp64"] = out["fp64"]["device_s"] / out["mixed"]["device_s"]
    print(json.dumps(out))


def time_to_residual(n, steps):
    """Poisson time-to-residual where the solve converges: the n x n cavity
    (Re 1000, omega 1.8, eps 1e-5 relative to each solve's starting norm),
    FP64 and mixed; per step the device time of the whole step (the solve
    dominates it) and the sweeps the solve took."""
    import torch
    from stroemung_gb300 import presets
    from stroemung_gb300.simulation import PREC_FP64, PREC_MIXED, ARITH_FAST, Simulation
    grid = presets.cavity(n)
    cfg = dict(cell_size=(1.0 / n, 1.0 / n), delt=1e-4, gamma=0.9, reynolds=1000.0,
               sor_absolute_epsilon=1e-5, max_iterations=100000, omega=1.8, tau=0.5,
               arithmetic=ARITH_FAST, strict_eps=2)
    out = {"grid": f"{n}x{n}", "stop_rule": "ns < (1e-5)^2 x the norm the solve starts from"}
    for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        sim = Simulation(grid=grid, precision=prec, **cfg)
        stream = torch.cuda.ExternalStream(sim.device_view()["stream"])
        rows = []
        for _ in range(steps):
            ms, st = timed_steps(sim, 1, stream)
            rows.append({"ms": ms, "sweeps": int(st[0][0]), "converged": bool(st[0][3])})
        sim.close()
        out[name] = {"per_step": rows,
                     "time_to_residual_ms_median": statistics.median(r["ms"] for r in rows)}
    out["speedup_mixed_vs_fp64"] = (out["fp64"]["time_to_residual_ms_median"] /
                                    out["mixed"]["time_to_residual_ms_median"])
    return out


def batch_specs(n: int):
    """n channel instances of uneven sizes (imax in 128..2048 step 128, jmax
    in 32..512 step 32, Re log-uniform in [50, 1000], 1..16 rectangles with
    the channel workload's placement rules), seeded; and their solver
    settings (mixed-precision members need ARITH_FAST here)."""
    import numpy as np
    from stroemung_gb300 import presets
    from stroemung_gb300.simulation import ARITH_FAST
    rng = np.random.default_rng(4)
    specs = []
    for k in range(n):
        imax = int(rng.integers(1, 17)) * 128
        jmax = int(rng.integers(1, 17)) * 32
        re = float(np.exp(rng.uniform(np.log(50.0), np.log(1000.0))))
        nrect = int(rng.integers(1, 17))
        side = (4, max(4, min(32, jmax // 4)))
        rects = presets.random_rectangles(imax, jmax, nrect, 1000 + k, side=side,
                                          x_margin=min(64, imax // 8))
        specs.append((presets.channel(imax, jmax, rects), re, imax * jmax))
    cfg = dict(cell_size=(0.01, 0.01), delt=0.005, gamma=0.9, sor_absolute_epsilon=1e-3,
               max_iterations=2000, omega=1.7, tau=0.5, arithmetic=ARITH_FAST)
    return specs, cfg


def batch_run(args):
    """--batch-run steps of the --batch-n channel instances as one batch, the
    members' mixed-precision solves as one persistent kernel per step, and in
    lockstep a second copy with the graph's WHILE loop; afterwards every
    member's u, v, p are compared bit for bit.  Then every instance one after
    another on the plain FP64 path (one warm step, one timed step each: the
    sequential baseline, which costs minutes per step over all instances).
    Prints one JSON document (not a benchmark line)."""
    import numpy as np
    import torch
    from stroemung_gb300.batch import Batch
    from stroemung_gb300.simulation import PREC_FP64, PREC_MIXED, Simulation
    specs, cfg = batch_specs(args.batch_n)
    cells = sum(c for _, _, c in specs)
    sets = {}
    for mode in ("persistent", "graph_loop"):
        sims = [Simulation(grid=g, reynolds=re, precision=PREC_MIXED, inner_sweeps=16, **cfg)
                for g, re, _ in specs]
        sets[mode] = (sims, Batch(sims))
    bp, bg = sets["persistent"][1], sets["graph_loop"][1]
    best, sched_ms = bg.autotune(reps=1)
    for b in (bp, bg):
        b.set_schedule(best)
    bp.set_solver(True)
    rows = {"persistent": [], "graph_loop": []}
    sweeps = []
    for step in range(args.batch_run):
        for mode, b in (("persistent", bp), ("graph_loop", bg)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = b.step(1)
            rows[mode].append(time.perf_counter() - t0)
            if mode == "persistent":
                sweeps.append(st["sor_iterations"][:, 0].astype(int))
    identical = True
    for a, b in zip(sets["persistent"][0], sets["graph_loop"][0]):
        for name in ("u", "v", "p"):
            if not np.array_equal(a.download(name), b.download(name)):
                identical = False
    for sims, b in sets.values():
        b.close()
        for sim in sims:
            sim.close()
    sw = np.array(sweeps)  # [step][member]
    t_seq, c_seq = 0.0, 0
    for g, re, c in specs:
        sim = Simulation(grid=g, reynolds=re, precision=PREC_FP64, **cfg)
        sim.run_simulation_tick()
        sim.synchronize()
        t0 = time.perf_counter()
        sim.step_n(1)
        t_seq += time.perf_counter() - t0
        c_seq += c
        sim.close()
    out = {"instances": len(specs), "cells": cells, "steps": args.batch_run,
           "sweep_schedule": best,
           "fields_identical_persistent_vs_graph_loop": identical,
           "sweeps_per_step_mean": [float(x) for x in sw.mean(axis=1)],
           "sweeps_total": int(sw.sum()),
           "sequential_fp64": {"value": c_seq / t_seq, "unit": "cell-updates/s",
                               "sample": "every instance, its second step (the first "
                                         "untimed), one after another"}}
    for mode, r in rows.items():
        out[mode] = {"s_total": sum(r), "value": cells * len(r) / sum(r),
                     "unit": "cell-updates/s", "ms_per_step_first": r[0] * 1e3,
                     "ms_per_step_median": statistics.median(r) * 1e3}
    out["steps_1_2_batch_vs_sequential_fp64"] = (
        cells * 2 / sum(rows["persistent"][:2])) / out["sequential_fp64"]["value"] \
        if len(rows["persistent"]) >= 2 else None
    print(json.dumps(out))


def batched_block(args):
    """Channel instances of uneven sizes (imax in 128..2048 step 128, jmax in
    32..512 step 32, Re log-uniform in [50, 1000], 1..16 rectangles), stepped
    as one batch vs one after another on the plain FP64 path."""
    import numpy as np
    import torch
    from stroemung_gb300 import presets
    from stroemung_gb300.batch import Batch
    from stroemung_gb300.simulation import PREC_FP64, PREC_MIXED, ARITH_FAST, Simulation
    specs, cfg = batch_specs(args.batch_n)
    cells = sum(c for _, _, c in specs)
    sims = [Simulation(grid=g, reynolds=re, precision=PREC_MIXED, inner_sweeps=16, **cfg)
            for g, re, _ in specs]
    batch = Batch(sims)
    batch.step(1)
    best, sched_ms = batch.autotune(reps=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = batch.step(args.batch_steps)
    torch.cuda.synchronize()
    t_batch = (time.perf_counter() - t0) / args.batch_steps
    # the same members' next steps with the solves as one persistent kernel
    batch.set_solver(True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st_p = batch.step(args.batch_steps)
    torch.cuda.synchronize()
    t_persist = (time.perf_counter() - t0) / args.batch_steps
    batch.close()
    for s in sims:
        s.close()
    learned = guarded_value(lambda: batched_learned(args, specs, cfg, best, st, t_batch)) \
        if args.batch_learned else None
    # the same instances one after another on the plain FP64 path (a sample,
    # scaled by cells)
    sample = list(range(0, len(specs), max(1, len(specs) // args.batch_seq_sample)))
    t_seq, c_seq = 0.0, 0
    for k in sample:
        g, re, c = specs[k]
        sim = Simulation(grid=g, reynolds=re, precision=PREC_FP64, **cfg)
        sim.run_simulation_tick()
        sim.synchronize()
        t0 = time.perf_counter()
        sim.step_n(1)
        t_seq += time.perf_counter() - t0
        c_seq += c
        sim.close()
    seq_rate = c_seq / t_seq
    rate = cells / t_batch
    return {
        "instances": len(specs), "cells": cells, "steps": args.batch_steps,
        "value": rate, "unit": "cell-updates/s", "ms_per_batch_step": t_batch * 1e3,
        "sequential_fp64": {"value": seq_rate, "unit": "cell-updates/s",
                            "sample_instances": len(sample)},
        "speedup_vs_sequential_fp64": rate / seq_rate,
        "sweep_schedule": {"chosen": best, "ms_per_batch_step": {str(k): v for k, v in
                                                                 sched_ms.items()}},
        "sor_iterations_mean": float(np.mean(st["sor_iterations"])),
        "persistent": {"value": cells / t_persist, "unit": "cell-updates/s",
                       "ms_per_batch_step": t_persist * 1e3,
                       "sor_iterations_mean": float(np.mean(st_p["sor_iterations"])),
                       "note": "the next steps of the same members with each step's "
                               "pressure solves as one persistent cooperative kernel"},
        "solver": "mixed precision (FP32 sweeps, FP64 norm/refinement), reference stop rule, "
                  "eps 1e-3, max_iterations 2000; one graph per step",
        "learned": learned,
    }


def guarded_value(fn):
    try:
        return fn()
    except Exception as exc:  # reported in the JSON line, not fatal
        return {"error": f"{type(exc).__name__}: {exc}"}


def batched_learned(args, specs, cfg, sched, st_plain, t_plain):
    """The same members with the learned warm start: a U-Net trained here on
    channel snapshots against their solved pressures (error loss), each
    member's prediction judged after 16 red-black iterations between the
    batch's halves; stepped from the state the plain batch's timed steps
    started from, so sweeps compare step by step."""
    import numpy as np
    import torch
    from stroemung_gb300 import warmstart
    from stroemung_gb300.batch import Batch
    from stroemung_gb300.simulation import PREC_MIXED, Simulation
    from stroemung_gb300.unet import UNet
    t0 = time.perf_counter()
    train = warmstart.generate_snapshots(args.batch_ws_snapshots, imax=512, jmax=128, dx=0.01,
                                         steps_per_problem=16, seed=11, targets=True)
    net = UNet(seed=0)
    tr = warmstart.Trainer(net, 514, 130, 0.01, 0.01, batch=32, loss="error")
    hist = tr.fit(train, epochs=args.batch_ws_epochs, lr=1e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del train
    sims = [Simulation(grid=g, reynolds=re, precision=PREC_MIXED, inner_sweeps=16, **cfg)
            for g, re, _ in specs]
    batch = Batch(sims)
    batch.set_schedule(sched)
    batch.step(1)
    bws = warmstart.BatchWarmStart(batch, net, judge_sweeps=args.ws_judge_sweeps)
    bws.warm_up()
    sweeps, acc = [], 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t_pj = 0.0
    for _ in range(args.batch_steps):
        rec = bws.step()
        sweeps.append(rec["sor_iterations"].astype(np.int64))
        acc += sum(bws.last["accepted"])
        t_pj += bws.last["predict_judge_s"]
    torch.cuda.synchronize()
    t_learned = (time.perf_counter() - t0) / args.batch_steps
    batch.close()
    for s in sims:
        s.close()
    plain = int(st_plain["sor_iterations"].astype(np.int64).sum())
    learned = int(np.sum(sweeps))
    return {"training": {"snapshots": args.batch_ws_snapshots, "grid": "512x128",
                         "epochs": args.batch_ws_epochs, "loss": "error",
                         "loss_first_last": [float(np.mean(hist[:8])),
                                             float(np.mean(hist[-8:]))],
                         "generate_and_train_s": t_train},
            "judge_sweeps": args.ws_judge_sweeps,
            "accepted": f"{acc}/{len(specs) * args.batch_steps}",
            "sweeps_plain": plain, "sweeps_learned": learned,
            "sweeps_saved": 1 - learned / plain,
            "ms_per_batch_step": t_learned * 1e3,
            "predict_and_judge_ms_per_batch_step": t_pj / args.batch_steps * 1e3,
            "time_vs_plain_batch": t_learned / t_plain}


def profile_target(what: str, steps: int) -> None:
    """Small workloads for ncu (no timing, no JSON): `fp64` / `mixed` run
    `steps` steps of the 4096 x 1024 channel with eager execution (every
    kernel a separate launch); `sweeps` runs 16 FP32 sweeps of the mixed
    solve after one step; `conv` runs two U-Net forwards at 4096 x 1024."""
    import torch
    from stroemung_gb300 import _lib
    from stroemung_gb300.simulation import PREC_FP64, PREC_MIXED, ARITH_FAST, Simulation
    if what == "conv":
        from stroemung_gb300.unet import UNet
        net = UNet(seed=0)
        x = torch.zeros(1, IMAX, JMAX, 8, dtype=torch.bfloat16, device="cuda")
        for _ in range(2):
            net.forward(x, 1, IMAX, JMAX)
        torch.cuda.synchronize()
        return
    prec = PREC_FP64 if what == "fp64" else PREC_MIXED
    sim = Simulation(grid=workload(SEED), precision=prec, arithmetic=ARITH_FAST,
                     execution=_lib.EXEC_EAGER if what != "sweeps" else _lib.EXEC_GRAPH,
                     **PARAMS)
    for _ in range(steps):
        print(sim.run_simulation_tick())
    if what == "sweeps":
        sim.sor_sweeps(16)
    sim.synchronize()
    sim.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--arith", default="fast", choices=["fast", "exact"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--ref-cap", type=int, default=10)
    ap.add_argument("--ref-parallel", type=int, default=1,
                    help="reference arm: also time the red-black order on every host core "
                         "(reported beside the single-core value)")
    ap.add_argument("--ref-full-steps", type=int, default=1,
                    help="reference arm: uncapped oracle ticks after the first, timed whole "
                         "beside the samples")
    ap.add_argument("--cpu-ticks", type=int, default=3)
    ap.add_argument("--cpu-cap", type=int, default=50)
    ap.add_argument("--eager", type=int, default=0,
                    help="1: launch kernels one by one (for per-kernel profiling)")
    ap.add_argument("--inner-sweeps", type=int, default=16)
    ap.add_argument("--inner-alt", type=int, nargs="*", default=[40, 80],
                    help="refinement intervals timed besides --inner-sweeps")
    ap.add_argument("--mixed", type=int, default=1)
    ap.add_argument("--err-steps", type=int, default=100,
                    help="steps after which mixed precision is compared with FP64")
    ap.add_argument("--full-steps", type=int, default=500,
                    help="steps of the whole-run block (FP64 and mixed from the start); 0 skips")
    ap.add_argument("--learned", type=int, default=1)
    ap.add_argument("--ws-weights", default="", help="trained U-Net parameters (.npy)")
    ap.add_argument("--ws-snapshots", type=int, default=1024)
    ap.add_argument("--ws-epochs", type=int, default=8)
    ap.add_argument("--ws-steps", type=int, default=4)
    ap.add_argument("--ws-cavity-n", type=int, default=128)
    ap.add_argument("--ws-cavity-epochs", type=int, default=30)
    ap.add_argument("--ws-cavity-steps", type=int, default=24)
    ap.add_argument("--ws-judge-sweeps", type=int, default=16)
    ap.add_argument("--cavity", type=int, default=1)
    ap.add_argument("--cavity-n", type=int, default=2048)
    ap.add_argument("--cavity-steps", type=int, default=3)
    ap.add_argument("--cavity-itermax", type=int, default=20000)
    ap.add_argument("--cavity-run", type=int, default=0,
                    help="run the cavity for this many steps, FP64 and mixed in lockstep, "
                         "and print a JSON report instead of the benchmark")
    ap.add_argument("--cavity-run-itermax", type=int, default=2000)
    ap.add_argument("--cavity-run-every", type=int, default=50)
    ap.add_argument("--cavity-small", type=int, default=256,
                    help="size of a cavity whose solves converge (time-to-residual); 0 skips")
    ap.add_argument("--batched", type=int, default=1)
    ap.add_argument("--batch-n", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=2)
    ap.add_argument("--batch-seq-sample", type=int, default=16)
    ap.add_argument("--batch-run", type=int, default=0,
                    help="step the batch this many steps, persistent and graph loop in "
                         "lockstep, and print a JSON report instead of the benchmark")
    ap.add_argument("--batch-learned", type=int, default=1,
                    help="also step the batch with the learned warm start")
    ap.add_argument("--batch-ws-snapshots", type=int, default=512)
    ap.add_argument("--batch-ws-epochs", type=int, default=20)
    ap.add_argument("--profile", default="", choices=["", "fp64", "mixed", "sweeps", "conv"],
                    help="run a small workload for ncu instead of the benchmark")
    args = ap.parse_args()
    if args.profile:
        profile_target(args.profile, max(args.steps if args.steps != 10 else 1, 1))
        return
    if args.cavity_run > 0:
        cavity_run(args)
        return
    if args.batch_run > 0:
        batch_run(args)
        return
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()

    from stroemung_gb300.simulation import ARITH_EXACT, ARITH_FAST, Simulation

    grid = workload(SEED + rank)
    arith = ARITH_FAST if args.arith == "fast" else ARITH_EXACT
    sim = Simulation(grid=grid, arithmetic=arith, execution=args.eager, **PARAMS)
    view = sim.device_view()
    stream = torch.cuda.ExternalStream(view["stream"])

    warm = sim.step_n(args.warmup)

    # ---- timed region: K steps, inputs resident ----
    with ClockSampler(local) as clocks:
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stats = sim.step_n(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), dist, "cuda")
    value = replica_value(CELLS, args.steps, world, ms / 1e3)
    iters = [s[0] for s in stats]
    if arith == ARITH_FAST:
        # boundary pass, F/G+RHS; copy + first red pass; the WHILE body of
        # FAST_BODY_ITERS black and red passes, run ceil((k + 1) /
        # FAST_BODY_ITERS) times for a solve that ends at iteration k (the
        # black pass of iteration k+1 applies k's stop test; the passes after
        # it return at once, but they are launched); the inverse of the last
        # red pass (omega away from 1) and the rollback; pressure range,
        # velocity
        unred = 1 if abs(1.0 - PARAMS["omega"]) >= 0.5 else 0
        launches = sum(2 + 2 + 2 * FAST_BODY_ITERS * -(-(k + 1) // FAST_BODY_ITERS)
                       + unred + 1 + 2 for k in iters)
    else:
        # per iteration copy, red, black, residual
        launches = sum(2 + 4 * k + 2 for k in iters)

    # ---- dominant kernel: the pressure iteration, timed live in the solve ----
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    sim.tick_prepare()
    sim.synchronize()
    s0.record(stream)
    n_solve, _ = sim.tick_solve()
    s1.record(stream)
    sim.synchronize()
    # the solve phase (one graph: the WHILE loop, then the velocity update,
    # < 0.1 % of it) divided by its iterations
    t_iter = s0.elapsed_time(s1) / 1e3 / max(n_solve, 1)
    interior = (IMAX) * (JMAX)
    sor_bytes = 25.0 * interior            # read p, rhs (16) + flags (1), write p (8)
    achieved = sor_bytes / t_iter / 1e9
    peak, peak_kind = load_peaks()
    # FP64 pipe work of one iteration: update on fluid cells + residual on all
    fluid = float((grid["kind"][1:-1, 1:-1] == 0).sum())
    # FAST: red update + the previous iteration's residual 7 and black update
    # + residual 7 per fluid cell of the colour, the residual of every other
    # interior cell 6 (the red fluid cells next to a wall pay 6 more)
    ops = (7.0 * fluid + 6 * (interior - fluid)) if arith == ARITH_FAST \
        else (17 * fluid + 20 * interior)
    fp64_peak = None
    try:
        a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        for _ in range(2):
            torch.matmul(a, a)
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record()
        for _ in range(5):
            torch.matmul(a, a)
        f1.record()
        torch.cuda.synchronize()
        fp64_peak = 2 * 4096 ** 3 * 5 / (f0.elapsed_time(f1) / 1e3) / 1e12
        del a
    except Exception:
        pass

    # ---- e2e: public API with host buffers, copies inside the timed region ----
    pin = {n: torch.empty((IMAX + 2, JMAX + 2), dtype=torch.float64, pin_memory=True)
           for n in ("u", "v", "p")}
    host = {n: pin[n].numpy() for n in pin}
    for n in host:
        sim.download(n, out=host[n])
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    e2e_iters = [0] if args.e2e_steps == 0 else []
    for _ in range(args.e2e_steps):
        for n in ("u", "v", "p"):
            sim.upload(n, host[n])
        e2e_iters.append(sim.run_simulation_tick()[0])
        for n in ("u", "v", "p"):
            sim.download(n, out=host[n])
    torch.cuda.synchronize()
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, "cuda")
    field_bytes = (IMAX + 2) * (JMAX + 2) * 8
    e2e = {"value": replica_value(CELLS, args.e2e_steps, world, e2e_s) if args.e2e_steps
           else None,
           "unit": "cell-updates/s",
           "h2d_bytes_per_step": 3 * field_bytes, "d2h_bytes_per_step": 3 * field_bytes + 64,
           "steps": args.e2e_steps, "sor_iterations": e2e_iters,
           "path": "Simulation.upload(u,v,p) + run_simulation_tick() + download(u,v,p), "
                   "pinned host buffers"}

    out = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded channel geometry, u = 1 start)", "config": config_dict(args),
        "sor_iterations": {"mean": statistics.mean(iters), "min": min(iters), "max": max(iters),
                           "warmup": [w[0] for w in warm]},
        "poisson": {"ms_per_step": 1e3 * t_iter * statistics.mean(iters),
                    "ms_per_iteration": 1e3 * t_iter,
                    "rule": "reference stop rule; no step reached eps" if not any(
                        s[3] for s in stats) else "reference stop rule"},
        "roofline": {"bound": "hbm", "kernel": "one red-black SOR iteration of the solve graph "
                     "(black pass + the black cells' residual + half the pressure copy, red "
                     "pass + the other half + the previous iteration's red cells' residual "
                     "and stop test)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes": sor_bytes,
                     # DRAM bytes of one iteration's kernels (red and black
                     # passes) in one ncu capture of this workload, cold cache
                     "traffic": SOR_ITERATION_TRAFFIC,
                     "traffic_note": "ncu dram__bytes read+write of one iteration's kernels, "
                                     "cold cache; each colour pass reads the whole of p and "
                                     "rhs (the colours interleave within cache lines); the "
                                     "updated pressures stay in the 129 MB L2 and are "
                                     "written back after the pass",
                     # the pipe that binds the FP64 iteration: its FP64
                     # operations per second against the FP64 instruction
                     # rate of a DGEMM measured here (2 FLOP per FMA)
                     "fp64_pipe_frac": (ops / t_iter) / (fp64_peak * 1e12 / 2) if fp64_peak
                     else None,
                     "fp64_pipe_note": "FP64 add/mul/fma instructions per second of the "
                                       "iteration over half the measured DGEMM FLOP rate (one "
                                       "FMA per two FLOP): the fraction of the FP64 pipe the "
                                       "iteration keeps busy"},
        "fp64": {"ops_per_iteration": ops, "achieved_tflops": ops / t_iter / 1e12,
                 "dgemm_tflops_measured": fp64_peak,
                 "pipe_ops_per_s_peak": fp64_peak * 1e12 / 2 if fp64_peak else None,
                 "note": "FP64 pipe operations (add, mul, fma each 1) of the solve"},
        "e2e": e2e,
        "clocks": clocks.summary(),
        "gpu_launches": launches,
    }
    if rank == 0 and world == 1 and args.cpu_ticks > 0:
        t_step, t_it, wall = cpu_sample(grid, statistics.mean(iters), args.cpu_ticks,
                                        args.cpu_cap)
        out["cpu_baseline"] = {
            "value": CELLS / t_step, "unit": "cell-updates/s", "cores": 1, "kind": "port",
            "sample": f"{args.cpu_ticks} oracle ticks of the same workload with the solve capped "
                      f"at {args.cpu_cap} iterations ({wall:.1f} s); step time = pre-solve + "
                      f"{statistics.mean(iters):.0f} (the GPU steps' mean) x per-iteration "
                      f"({t_it * 1e3:.1f} ms) + post-solve",
            "host_cpu": os.uname().machine, "nproc": os.cpu_count()}

    if rank == 0:
        fp64_ms_step = ms / args.steps
        mixed_ms = None

        def guarded(name, fn):
            # an auxiliary block that fails is reported, not fatal to the line
            try:
                out[name] = fn()
            except Exception as exc:  # noqa: BLE001
                out[name] = {"error": f"{type(exc).__name__}: {exc}"}
            torch.cuda.empty_cache()

        sim.close()
        sim = None
        if args.mixed:
            guarded("mixed_precision", lambda: mixed_block(args, grid, fp64_ms_step, peak))
            mixed_ms = out["mixed_precision"].get("ms_per_step")
        if args.full_steps > 0:
            guarded("full_run", lambda: full_run_block(args, grid))
        if args.learned:
            guarded("learned", lambda: learned_block(args, grid, fp64_ms_step, mixed_ms))
            guarded("learned_cavity", lambda: learned_cavity_block(args))
        if args.cavity:
            guarded("cavity_mixed", lambda: cavity_block(args))
        if args.batched:
            guarded("batched", lambda: batched_block(args))
        print(json.dumps(out))
    if sim is not None:
        sim.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
