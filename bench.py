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
steps / device time), inputs resident in HBM; `e2e` is the same metric
through the public API with host (pinned) buffers uploaded and downloaded
every step.  Under torchrun each rank runs its own replica (weak scaling).
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
L2_BYTES = 129e6


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


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


def cpu_sample(grid, k_iters: float, ticks: int, cap: int):
    """Times the oracle on the host: `ticks` ticks of the full workload with the
    solve capped at `cap` iterations; returns the per-step time for a step of
    k_iters iterations (phase times measured, iterations scaled)."""
    from oracle import oracle as orc
    orc.build()
    p = PARAMS
    o = orc.OracleSim(kind=grid["kind"], wall_uv=grid["wall_uv"], u=grid["u"], v=grid["v"],
                      p=grid["p"], dx=p["cell_size"][0], dy=p["cell_size"][1], delt=p["delt"],
                      gamma=p["gamma"], reynolds=p["reynolds"], eps=p["sor_absolute_epsilon"],
                      omega=p["omega"], max_iterations=p["max_iterations"], tau=p["tau"])
    pre, it_s, post = [], [], []
    t0 = time.perf_counter()
    for _ in range(ticks):
        a, b, n, c = o.tick_timed(cap)
        pre.append(a)
        post.append(c)
        if n > 0:
            it_s.append(b / n)
    wall = time.perf_counter() - t0
    t_iter = statistics.mean(it_s) if it_s else 0.0
    t_step = statistics.mean(pre) + k_iters * t_iter + statistics.mean(post)
    return t_step, t_iter, wall


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    grid = workload(SEED)
    k = PARAMS["max_iterations"]
    times = []
    for i in range(args.warmup + args.steps):
        t_step, t_iter, _ = cpu_sample(grid, k, 1, args.ref_cap)
        if i >= args.warmup:
            times.append(t_step)
    t = statistics.mean(times)
    value = CELLS / t
    sample = (f"each step: one oracle tick of the full 4096x1024 workload with the pressure "
              f"solve capped at {args.ref_cap} iterations; step time = measured pre-solve + "
              f"{k} x measured per-iteration + measured post-solve time ({k} = "
              f"max_iterations, what this configuration's solve runs per step)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_dict(args),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": 1, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }))


METRIC = "cell-updates/s (4096x1024 channel timestep, FP64 red-black SOR)"


def config_dict(args):
    return {"workload": "channel 4096x1024, 64 rectangles (seed 0), Re 400, tau 0.5, "
                        "eps 1e-3, max_iterations 2000",
            "imax": IMAX, "jmax": JMAX, "obstacles": NRECTS,
            "solver": f"red-black SOR, FP64, {args.arith} arithmetic",
            "stop_rule": "reference (ns < initial norm or ns < eps^2)",
            "l2": "per-step working set (9 FP64 fields + flags, 285 MB) exceeds the 129 MB L2; "
                  "no flush", "parallelism": f"replicas x{args.gpus}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--arith", default="fast", choices=["fast", "exact"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--ref-cap", type=int, default=10)
    ap.add_argument("--cpu-ticks", type=int, default=3)
    ap.add_argument("--cpu-cap", type=int, default=50)
    ap.add_argument("--mixed", type=int, default=1)
    ap.add_argument("--eager", type=int, default=0,
                    help="1: launch kernels one by one (for per-kernel profiling)")
    ap.add_argument("--inner-sweeps", type=int, default=16)
    args = ap.parse_args()
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
    ms = e0.elapsed_time(e1)
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = CELLS * args.steps * world / (ms / 1e3)
    iters = [s[0] for s in stats]
    n_pcopy_launch = 1
    launches = sum(2 + 3 + n_pcopy_launch + (3 + n_pcopy_launch) * (k - 1) + 2 for k in iters)
    fp64_fields = {n: sim.download(n) for n in ("u", "v", "p")}

    # ---- dominant kernel: one red-black iteration, timed live ----
    nsweep = 20
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    sim.synchronize()
    s0.record(stream)
    sim.sor_sweeps(nsweep, wait=False)
    s1.record(stream)
    sim.synchronize()
    t_iter = s0.elapsed_time(s1) / 1e3 / nsweep
    interior = (IMAX) * (JMAX)
    sor_bytes = 25.0 * interior            # read p, rhs (16) + flags (1), write p (8)
    achieved = sor_bytes / t_iter / 1e9
    peak, peak_kind = load_peaks()
    # FP64 pipe work of one iteration: update on fluid cells + residual on all
    fluid = float((grid["kind"][1:-1, 1:-1] == 0).sum())
    ops = (6 if arith == ARITH_FAST else 17) * fluid + (7 if arith == ARITH_FAST else 20) * interior
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

    # ---- mixed precision on the same workload: FP32 sweeps, FP64 norm and
    # refinement; same warm-up and timed steps from the same initial state ----
    mixed = None
    if args.mixed:
        from stroemung_gb300.simulation import PREC_MIXED
        simm = Simulation(grid=grid, precision=PREC_MIXED, inner_sweeps=args.inner_sweeps,
                          execution=args.eager, **PARAMS)
        stream_m = torch.cuda.ExternalStream(simm.device_view()["stream"])
        warm_m = simm.step_n(args.warmup)
        torch.cuda.synchronize()
        m0 = torch.cuda.Event(enable_timing=True)
        m1 = torch.cuda.Event(enable_timing=True)
        m0.record(stream_m)
        stats_m = simm.step_n(args.steps)
        m1.record(stream_m)
        torch.cuda.synchronize()
        ms_m = m0.elapsed_time(m1)
        iters_m = [x[0] for x in stats_m]
        err = {}
        fl = grid["kind"] == 0
        for n in ("u", "v", "p"):
            a, b = simm.download(n), fp64_fields[n]
            if n == "p":  # pressure is defined up to a constant: fluid cells, mean removed
                a, b = a[fl] - a[fl].mean(), b[fl] - b[fl].mean()
            err[n] = {"rel_l2": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)),
                      "max_abs": float(np.abs(a - b).max())}
        sw0 = torch.cuda.Event(enable_timing=True)
        sw1 = torch.cuda.Event(enable_timing=True)
        simm.synchronize()
        sw0.record(stream_m)
        simm.sor_sweeps(nsweep, wait=False)
        sw1.record(stream_m)
        simm.synchronize()
        t_sw = sw0.elapsed_time(sw1) / 1e3 / nsweep
        sw_bytes = 13.0 * interior  # read e, s (8) + flags (1), write e (4)
        m_inner = min(args.inner_sweeps, PARAMS["max_iterations"])
        mixed = {
            "value": CELLS * args.steps * world / (ms_m / 1e3), "unit": "cell-updates/s",
            "ms_per_step": ms_m / args.steps, "speedup_vs_fp64": ms / ms_m,
            "inner_sweeps": m_inner,
            "sor_iterations": {"mean": statistics.mean(iters_m), "min": min(iters_m),
                               "max": max(iters_m), "warmup": [w[0] for w in warm_m]},
            "error_vs_fp64_after_steps": {"steps": args.warmup + args.steps, **err},
            "roofline_fp32_sweep": {"achieved": sw_bytes / t_sw / 1e9, "peak": peak,
                                    "unit": "GB/s", "frac": sw_bytes / t_sw / 1e9 / peak,
                                    "ms_per_sweep": t_sw * 1e3,
                                    "algorithmic_bytes": sw_bytes},
            "dtype": "f32 sweeps, f64 norm/refinement/dt",
        }
        simm.close()

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
    e2e_s = time.perf_counter() - t0
    if dist is not None:
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    field_bytes = (IMAX + 2) * (JMAX + 2) * 8
    e2e = {"value": CELLS * args.e2e_steps * world / e2e_s if args.e2e_steps else None, "unit": "cell-updates/s",
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
        "roofline": {"bound": "hbm", "kernel": "one red-black SOR iteration "
                     "(pressure copy + red + black + residual)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "algorithmic_bytes": sor_bytes, "traffic": None},
        "fp64": {"ops_per_iteration": ops, "achieved_tflops": ops / t_iter / 1e12,
                 "dgemm_tflops_measured": fp64_peak,
                 "note": "FP64 pipe operations (add, mul, fma each 1) of the solve"},
        "e2e": e2e,
        "mixed_precision": mixed,
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
        print(json.dumps(out))
    sim.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
