"""Learned warm start for the pressure solve: snapshot generation, training
and the in-the-loop predictor with plain SOR as judge and fallback.

Snapshots come from the solver itself: seeded problems (channels with the
benchmark's obstacle placement rules, or lid-driven cavities), each stepped
with ``tick_prepare`` / ``tick_solve``; between the two the step's RHS, the
previous pressure and the flags are exported (FP32 / u8, full [nx][ny]
planes) — the network's input — and, when targets are asked for, the
pressure the solve reached afterwards (the training target of the error
loss).

Two losses: ``residual`` (the relative Poisson residual of the corrected
pressure, Σr²/Σrhs²) and ``error`` (the relative error against the solved
pressure, both mean-free on fluid cells).  Measured: the residual loss
learns to remove the rough part of the error, which the first SOR sweeps
remove anyway, and saves no sweeps; the error loss learns the smooth part,
which is what SOR is slow on.

In the loop (``WarmStartSolver.step``): after ``tick_prepare`` the network
predicts a correction q; ``strm_judge_correction`` keeps p_prev + s*dx^2*q
only if it beats p_prev on the solver's own norm — right away (judge_sweeps
0: the initial residual) or after judge_sweeps red-black iterations of both
(a smooth correction with a little rough error has the larger raw residual)
— then ``tick_solve`` runs the unchanged solve to the same stop rule.
"""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from . import _lib, presets
from .unet import IN_CH, UNet


class PlaneBatch:
    """Device planes for `batch` samples of one grid size (target: the
    solved pressure of each sample, allocated on request)."""

    def __init__(self, batch, nx, ny, device="cuda", targets=False):
        import torch
        self.batch, self.nx, self.ny = batch, nx, ny
        self.rhs = torch.zeros(batch, nx, ny, dtype=torch.float32, device=device)
        self.p = torch.zeros(batch, nx, ny, dtype=torch.float32, device=device)
        self.flags = torch.zeros(batch, nx, ny, dtype=torch.uint8, device=device)
        self.target = (torch.zeros(batch, nx, ny, dtype=torch.float32, device=device)
                       if targets else None)


def export_sample(sim, planes: PlaneBatch, i: int):
    """Copies sim's current RHS, pressure and flags into sample i."""
    off = i * planes.nx * planes.ny
    _lib.check(_lib.load().strm_export_planes(
        sim._h, planes.rhs.data_ptr() + 4 * off, planes.p.data_ptr() + 4 * off,
        planes.flags.data_ptr() + off))


def export_target(sim, planes: PlaneBatch, i: int):
    """Copies sim's pressure (after the solve) into sample i's target."""
    off = i * planes.nx * planes.ny
    _lib.check(_lib.load().strm_export_planes(sim._h, None, planes.target.data_ptr() + 4 * off,
                                              None))


def channel_problem(rng, imax, jmax, seed, nrect=None, re=None):
    """A seeded channel with rectangular obstacles (the benchmark's placement
    rules; 4..32 rectangles of side 4..32 cells at 512 x 128, fewer and
    smaller on smaller grids) and a Reynolds number log-uniform in [50, 1000]."""
    re = float(np.exp(rng.uniform(math.log(50.0), math.log(1000.0)))) if re is None else re
    hi = min(32, max(4, imax * jmax // 2048))
    nrect = int(rng.integers(min(4, hi), hi + 1)) if nrect is None else nrect
    side = (4, max(4, min(32, jmax // 4)))
    margin = min(64, imax // 8)
    rects = presets.random_rectangles(imax, jmax, nrect, seed, side=side, x_margin=margin)
    return presets.channel(imax, jmax, rects), re


SOLVER = {"sor_absolute_epsilon": 1e-3, "max_iterations": 2000, "omega": 1.7, "tau": 0.5,
          "gamma": 0.9}


def make_simulation(grid, re, dx, **solver):
    """A Simulation with the solver settings the warm start uses: mixed
    precision, strict eps on the mean-free fluid-cell residual."""
    from .simulation import NORM_FLUID_MEAN_FREE, PREC_MIXED, Simulation
    cfg = dict(SOLVER)
    cfg.update(solver)
    mode = {"precision": PREC_MIXED, "strict_eps": True, "norm_cells": NORM_FLUID_MEAN_FREE}
    for k in ("precision", "strict_eps", "norm_cells", "inner_sweeps", "arithmetic",
              "sweep_schedule"):
        if k in cfg:
            mode[k] = cfg.pop(k)
    delt = cfg.pop("delt", 0.5 * dx)
    return Simulation(grid=grid, cell_size=(dx, dx), delt=delt, reynolds=re, **cfg, **mode)


def channel_family(imax=512, jmax=128, dx=0.01):
    """Problem family: seeded channels (the benchmark's geometry rules)."""
    def make(rng, seed, **solver):
        grid, re = channel_problem(rng, imax, jmax, seed)
        return make_simulation(grid, re, dx, **solver)
    return make, (imax + 2, jmax + 2)


def cavity_family(n=128, re_range=(50.0, 2000.0)):
    """Problem family: n x n lid-driven cavities, unit square, Reynolds
    number log-uniform in re_range."""
    def make(rng, seed, **solver):
        re = float(np.exp(rng.uniform(math.log(re_range[0]), math.log(re_range[1]))))
        cfg = dict(delt=1e-3, max_iterations=40000)
        cfg.update(solver)
        return make_simulation(presets.cavity(n), re, 1.0 / n, **cfg)
    return make, (n + 2, n + 2)


def generate_snapshots(n_snapshots, imax=512, jmax=128, dx=0.01, steps_per_problem=25,
                       seed=0, device="cuda", family=None, targets=False, **solver):
    """Runs seeded problems (channels of imax x jmax unless `family` is given)
    and returns a PlaneBatch with one sample per step (RHS, previous
    pressure, flags, and with targets the solved pressure)."""
    make, (nx, ny) = family if family is not None else channel_family(imax, jmax, dx)
    planes = PlaneBatch(n_snapshots, nx, ny, device, targets=targets)
    rng = np.random.default_rng(seed)
    i = 0
    k = 0
    while i < n_snapshots:
        sim = make(rng, seed * 100003 + k, **solver)
        k += 1
        for _ in range(steps_per_problem):
            if i >= n_snapshots:
                break
            sim.tick_prepare()
            export_sample(sim, planes, i)
            sim.tick_solve()
            if targets:
                export_target(sim, planes, i)
            i += 1
        sim.close()
    return planes


class Trainer:
    """Adam on the relative Poisson residual of the corrected pressure
    (loss="residual") or on its relative error against the solved pressure
    (loss="error", planes with targets)."""

    def __init__(self, net: UNet, nx, ny, dx, dy, batch=32, loss="residual"):
        import torch
        if loss not in ("residual", "error"):
            raise ValueError(loss)
        self.kind = loss
        self.net, self.nx, self.ny, self.batch = net, nx, ny, batch
        self.dx2 = dx * dx
        self.rdx2, self.rdy2 = 1.0 / (dx * dx), 1.0 / (dy * dy)
        dev = net.device
        h, w = nx - 2, ny - 2
        self.xin = torch.zeros(batch, h, w, IN_CH, dtype=torch.bfloat16, device=dev)
        self.smax = torch.zeros(batch, dtype=torch.float32, device=dev)
        self.pmean = torch.zeros(batch, dtype=torch.float32, device=dev)
        self.work2 = torch.zeros(2 * batch, dtype=torch.float32, device=dev)
        self.pfull = torch.zeros(batch, nx, ny, dtype=torch.float32, device=dev)
        self.r = torch.zeros(batch, nx, ny, dtype=torch.float32, device=dev)
        self.gp = torch.zeros(batch, nx, ny, dtype=torch.float32, device=dev)
        self.gq = torch.zeros(batch, h, w, dtype=torch.float32, device=dev)
        self.sum_r2 = torch.zeros(batch, dtype=torch.float32, device=dev)
        self.sum_b2 = torch.zeros(batch, dtype=torch.float32, device=dev)
        self.work5 = torch.zeros(5 * batch, dtype=torch.float32, device=dev)
        self.per = torch.zeros(batch, dtype=torch.float32, device=dev)

    def _planes(self, planes: PlaneBatch, start):
        off = start * self.nx * self.ny
        return (planes.rhs.data_ptr() + 4 * off, planes.flags.data_ptr() + off,
                planes.p.data_ptr() + 4 * off)

    def loss(self, planes: PlaneBatch, start, batch=None, grad=False):
        """Mean loss of samples [start, start+batch) after the network's
        correction and the per-sample values (grad: also the gradient with
        respect to q into self.gq)."""
        b = self.batch if batch is None else batch
        L = self.net.L
        rhs, flags, pprev = self._planes(planes, start)
        h, w = self.nx - 2, self.ny - 2
        self.net._check(L.strm_nn_prepare_input(rhs, flags, pprev, self.smax.data_ptr(),
                                                self.pmean.data_ptr(), self.work2.data_ptr(),
                                                self.dx2, self.xin.data_ptr(), b, self.nx,
                                                self.ny, None), "prepare")
        q = self.net.forward(self.xin, b, h, w)
        if self.kind == "error":
            off = start * self.nx * self.ny
            self.net._check(L.strm_nn_error_loss(
                pprev, q.data_ptr(), planes.target.data_ptr() + 4 * off, flags,
                self.smax.data_ptr(), self.dx2, self.work5.data_ptr(), self.per.data_ptr(),
                self.gq.data_ptr() if grad else None, b, self.nx, self.ny, None), "error loss")
            per = self.per[:b].detach().cpu().numpy()
            return float(per.mean()), per
        self.net._check(L.strm_nn_residual_loss(pprev, q.data_ptr(), flags, rhs,
                                                self.smax.data_ptr(), self.dx2, self.rdx2,
                                                self.rdy2, self.pfull.data_ptr(),
                                                self.r.data_ptr(), self.sum_r2.data_ptr(),
                                                self.sum_b2.data_ptr(), b, self.nx, self.ny,
                                                None), "loss")
        if grad:
            self.net._check(L.strm_nn_residual_loss_grad(
                self.r.data_ptr(), flags, self.sum_b2.data_ptr(), self.smax.data_ptr(),
                self.dx2, self.rdx2, self.rdy2, self.gp.data_ptr(), self.gq.data_ptr(), b,
                self.nx, self.ny, None), "loss grad")
        per = (self.sum_r2[:b] / self.sum_b2[:b].clamp_min(1e-30)).detach().cpu().numpy()
        return float(per.mean()), per

    def train_step(self, planes: PlaneBatch, start, lr=1e-3):
        b = self.batch
        loss, _ = self.loss(planes, start, grad=True)
        self.net.zero_grad()
        self.net.backward(self.gq, b, self.nx - 2, self.ny - 2)
        self.net.adam(lr=lr)
        return loss

    def fit(self, planes: PlaneBatch, epochs=1, lr=1e-3, log=None, seed=0, max_steps=None):
        n = planes.batch
        rng = np.random.default_rng(seed)
        history = []
        steps = 0
        for ep in range(epochs):
            starts = rng.permutation(n // self.batch) * self.batch
            for s0 in starts:
                history.append(self.train_step(planes, int(s0), lr))
                steps += 1
                if max_steps and steps >= max_steps:
                    return history
            if log:
                log(f"epoch {ep}: loss {np.mean(history[-len(starts):]):.4e}")
        return history


class WarmStartSolver:
    """A Simulation stepped with the learned warm start: after tick_prepare
    the network predicts a correction of the previous pressure; the
    corrected pressure is kept only if its residual norm (the solver's norm
    after the boundary copy) is below the previous pressure's, else the
    previous pressure is restored (plain SOR is judge and fallback); then
    tick_solve runs the unchanged solve from there."""

    def __init__(self, sim, net: UNet, judge_sweeps: int = 0, graphed: bool = True):
        import torch
        self.sim, self.net = sim, net
        self.judge_sweeps = int(judge_sweeps)
        self.graphed = bool(graphed)  # replay the network's forward from a CUDA graph
        nx, ny = sim.size
        self.planes = PlaneBatch(1, nx, ny, net.device)
        self.trainer = Trainer(net, nx, ny, sim.cell_size[0], sim.cell_size[1], batch=1)
        self.accepted = 0
        self.rejected = 0
        self.last = {}

    def predict(self):
        """Network correction q [nx-2][ny-2] (device FP32) of the prepared
        step and its scale s * dx^2."""
        import torch
        L = _lib.load()
        export_sample(self.sim, self.planes, 0)
        tr = self.trainer
        rhs, flags, pprev = tr._planes(self.planes, 0)
        self.net._check(L.strm_nn_prepare_input(rhs, flags, pprev, tr.smax.data_ptr(),
                                                tr.pmean.data_ptr(), tr.work2.data_ptr(),
                                                tr.dx2, tr.xin.data_ptr(), 1, tr.nx, tr.ny,
                                                None), "prepare")
        if self.graphed:
            q = self.net.forward_graphed(tr.xin, 1, tr.nx - 2, tr.ny - 2)
        else:
            q = self.net.forward(tr.xin, 1, tr.nx - 2, tr.ny - 2, keep=False)
        torch.cuda.synchronize()
        return q, float(tr.smax[0].item()) * tr.dx2

    def warm_up(self):
        """Records the predictor's graph now (the first prediction does it
        otherwise); the simulation's state is not changed."""
        if self.graphed:
            self.predict()

    def judge(self, q, scale):
        """Keeps the correction if it beats the previous pressure on the
        solver's norm (after judge_sweeps red-black iterations of both;
        judge_sweeps < 0 takes it unjudged); returns (accepted, norm
        without, norm with the correction)."""
        if self.judge_sweeps < 0:  # no judge: always take the prediction
            _lib.check(_lib.load().strm_apply_correction(self.sim._h, q.data_ptr(), scale))
            self.sim.copy_pressure_to_boundaries()
            self.accepted += 1
            return True, float("nan"), float("nan")
        a, b = ctypes.c_double(0.0), ctypes.c_double(0.0)
        acc = ctypes.c_int(0)
        _lib.check(_lib.load().strm_judge_correction(
            self.sim._h, q.data_ptr(), scale, self.judge_sweeps, ctypes.byref(a),
            ctypes.byref(b), ctypes.byref(acc)))
        if acc.value:
            self.accepted += 1
        else:
            self.rejected += 1
        return bool(acc.value), a.value, b.value

    def step(self):
        t0 = time.perf_counter()
        self.sim.tick_prepare()
        q, scale = self.predict()
        t1 = time.perf_counter()
        accepted, ns_prev, ns_pred = self.judge(q, scale)
        t2 = time.perf_counter()
        it, ns = self.sim.tick_solve()
        self.last = {"ns_prev": ns_prev, "ns_pred": ns_pred, "accepted": accepted,
                     "predict_s": t1 - t0, "judge_s": t2 - t1,
                     "solve_s": time.perf_counter() - t2}
        return it, ns


class BatchWarmStart:
    """The learned warm start for a Batch: between the batch's two halves
    every member's pressure is predicted and judged as WarmStartSolver does
    for one simulation; then the members' pressure solves run together in
    the batch's WHILE loop.  Each member ends exactly where its own
    WarmStartSolver steps would end."""

    def __init__(self, batch, net: UNet, judge_sweeps: int = 16):
        self.batch = batch
        self.members = [WarmStartSolver(s, net, judge_sweeps) for s in batch.sims]
        self.last = {}

    def warm_up(self):
        """Records every member's predictor graph now.  Two passes: a member
        whose forward needs a larger pool than the earlier ones drops their
        recordings, and the second pass finds the pool at its final size."""
        for _ in range(2):
            for w in self.members:
                w.warm_up()

    def step(self):
        """One batch step; returns the per-member records of Batch.solve and
        keeps the accepted flags and the predictor/judge time in self.last."""
        import torch
        self.batch.prepare()
        t0 = time.perf_counter()
        accepted = []
        for w in self.members:
            q, scale = w.predict()
            accepted.append(w.judge(q, scale)[0])
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        out = self.batch.solve()
        self.last = {"accepted": accepted, "predict_judge_s": t1 - t0,
                     "solve_s": time.perf_counter() - t1}
        return out


def sync_state(dst, src, scratch):
    """Copies u, v and p of simulation src into dst (device to device)."""
    L = _lib.load()
    for f in (_lib.FIELD_U, _lib.FIELD_V, _lib.FIELD_P):
        _lib.check(L.strm_copy_field_device(src._h, f, scratch.data_ptr(), 0))
        _lib.check(L.strm_copy_field_device(dst._h, f, scratch.data_ptr(), 1))


def sweeps_to_reach(history, target):
    """First sweep count at which a (sweeps, norm) history is <= target, or None."""
    for sw, ns in history:
        if ns <= target:
            return int(sw)
    return None


def compare_step(plain, ws: WarmStartSolver, scratch):
    """One step of the same state solved twice: `plain` from the previous
    pressure, `ws` from the judged prediction; afterwards ws takes plain's
    fields so that the next step starts from identical states again.
    Returns the per-step record (norm histories, sweeps to plain's final
    norm, predictor time)."""
    import torch
    plain.tick_prepare()
    ws.sim.tick_prepare()
    t0 = time.perf_counter()
    q, scale = ws.predict()
    t1 = time.perf_counter()
    accepted, ns_prev, ns_pred = ws.judge(q, scale)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    t3 = time.perf_counter()
    it_p, ns_p = plain.tick_solve()
    t4 = time.perf_counter()
    it_w, ns_w = ws.sim.tick_solve()
    t5 = time.perf_counter()
    hp, hw = plain.residual_history(), ws.sim.residual_history()
    sync_state(ws.sim, plain, scratch)
    return {"sweeps_plain": it_p, "sweeps_ws": it_w, "ns_plain": ns_p, "ns_ws": ns_w,
            "ns0_plain": float(hp[0, 1]), "ns0_ws": float(hw[0, 1]), "accepted": accepted,
            "ns_prev": ns_prev, "ns_pred": ns_pred,
            "ws_sweeps_to_plain_final": sweeps_to_reach(hw, ns_p),
            "predict_ms": (t1 - t0) * 1e3, "judge_ms": (t2 - t1) * 1e3,
            "solve_plain_ms": (t4 - t3) * 1e3, "solve_ws_ms": (t5 - t4) * 1e3,
            "hist_plain": hp, "hist_ws": hw}
