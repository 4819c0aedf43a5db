"""Batches: every member of a batch step ends bit-identical to the same
simulation stepped alone (fields, iteration counts, norms, time steps),
with members of different sizes, Reynolds numbers and stop rules, some of
which stop early while others run to max_iterations."""
import numpy as np
import pytest

from stroemung_gb300 import _lib, presets
from stroemung_gb300.batch import Batch
from stroemung_gb300.simulation import (NORM_FLUID_MEAN_FREE, PREC_MIXED, Simulation,
                                        StroemungError)

pytestmark = pytest.mark.gpu


def _members():
    """(grid, kwargs): channels of several sizes and a closed cavity that
    converges under the strict mean-free rule."""
    out = []
    for k, (imax, jmax, nrect, re) in enumerate([(128, 32, 1, 80.0), (256, 96, 3, 400.0),
                                                  (384, 64, 2, 900.0)]):
        rects = presets.random_rectangles(imax, jmax, nrect, 10 + k, side=(4, 12), x_margin=16)
        out.append((presets.channel(imax, jmax, rects),
                    dict(reynolds=re, max_iterations=160 + 32 * k)))
    cav = dict(reynolds=100.0, max_iterations=400, strict_eps=True,
               norm_cells=NORM_FLUID_MEAN_FREE, sor_absolute_epsilon=1e-12)
    # eps such that the first step of the cavity stops after about 160 sweeps
    probe = _make(presets.cavity(48), cav, 3)
    probe.run_simulation_tick()
    hist = probe.residual_history()
    probe.close()
    target = hist[hist[:, 0] <= 160][-1, 1]
    cav["sor_absolute_epsilon"] = float(np.sqrt(target * 1.0001))
    out.append((presets.cavity(48), cav))
    return out


def _make(grid, kw, schedule):
    cfg = dict(cell_size=(0.01, 0.01), delt=0.002, gamma=0.9, sor_absolute_epsilon=1e-3,
               omega=1.7, tau=0.5, precision=PREC_MIXED, sweep_schedule=schedule)
    cfg.update(kw)
    return Simulation(grid=grid, **cfg)


@pytest.mark.parametrize("schedule", [3, 6])
def test_batch_members_match_single_runs_bitwise(schedule):
    steps = 5
    members = _members()
    alone = []
    for grid, kw in members:
        sim = _make(grid, kw, schedule)
        stats = [sim.run_simulation_tick() for _ in range(steps)]
        alone.append((stats, {k: sim.download(k) for k in ("u", "v", "p")}, sim.state()))
        sim.close()
    sims = [_make(grid, kw, schedule) for grid, kw in members]
    with Batch(sims) as batch:
        batch.set_schedule(schedule)
        st = batch.step(steps)
    for k, sim in enumerate(sims):
        stats, fields, state = alone[k]
        assert [int(x) for x in st[k]["sor_iterations"]] == [s[0] for s in stats], k
        assert list(st[k]["norm_squared"]) == [s[1] for s in stats], k
        for name in fields:
            np.testing.assert_array_equal(sim.download(name), fields[name],
                                          err_msg=f"member {k} field {name}")
        assert sim.state()["time"] == state["time"]
    # the cavity stopped early, the channels ran to their limits
    assert st[3]["converged"].any() and not st[0]["converged"].any()
    for s in sims:
        s.close()


def test_batch_continues_member_state_and_autotunes():
    members = _members()[:2]
    sims = [_make(g, kw, 3) for g, kw in members]
    ref = [_make(g, kw, 3) for g, kw in members]
    for r in ref:
        for _ in range(4):
            r.run_simulation_tick()
    # two steps alone, then two in a batch (after an autotune that restores state)
    for s in sims:
        for _ in range(2):
            s.run_simulation_tick()
    with Batch(sims) as batch:
        best, times = batch.autotune(reps=1)
        assert 2 <= best < _lib.SWEEPS_COUNT and times[best] == min(times.values())
        batch.set_schedule(3)
        batch.step(2)
    for s, r in zip(sims, ref):
        for name in ("u", "v", "p"):
            np.testing.assert_array_equal(s.download(name), r.download(name))
        s.close()
        r.close()


def test_batch_rejects_unsuitable_members():
    grid, kw = _members()[0]
    fp64 = Simulation(grid=grid, cell_size=(0.01, 0.01), delt=0.002, gamma=0.9, reynolds=100.0,
                      max_iterations=50)
    with pytest.raises(StroemungError):
        Batch([fp64])
    short = _make(grid, dict(reynolds=100.0, max_iterations=8), 3)
    with pytest.raises(StroemungError):
        Batch([short])
    fp64.close()
    short.close()


def test_batch_halves_equal_batch_steps():
    """prepare + solve, three times, gives the fields and records of
    step(3)."""
    members = _members()
    a = [_make(g, kw, 3) for g, kw in members]
    b = [_make(g, kw, 3) for g, kw in members]
    with Batch(a) as ba, Batch(b) as bb:
        st = ba.step(3)
        for i in range(3):
            bb.prepare()
            rec = bb.solve()
            for k in range(len(b)):
                assert rec[k]["sor_iterations"] == st[k, i]["sor_iterations"]
                assert rec[k]["norm_squared"] == st[k, i]["norm_squared"]
                assert rec[k]["delt"] == st[k, i]["delt"]
    for sa, sb in zip(a, b):
        for n in ("u", "v", "p"):
            np.testing.assert_array_equal(sb.download(n), sa.download(n), err_msg=n)
        sa.close()
        sb.close()


def _net_with_random_head(seed=3):
    import torch
    from stroemung_gb300.unet import UNet
    net = UNet(seed=seed)
    th = net.theta.detach().cpu().numpy().copy()
    th[-33:] = np.random.default_rng(seed).normal(0.0, 0.3, 33).astype(np.float32)
    net.load_state_dict({"theta": th, "step": 0})
    torch.cuda.synchronize()
    return net


@pytest.mark.parametrize("judge_sweeps", [-1, 4])
def test_batch_warm_start_matches_members_stepped_alone(judge_sweeps):
    """A batch stepped with the learned warm start (prediction and judge per
    member between the batch's halves) ends bit-identical to each member
    stepped alone by WarmStartSolver; judge -1 applies every prediction."""
    from stroemung_gb300 import warmstart
    net = _net_with_random_head()
    members = _members()
    steps = 3
    alone = []
    for grid, kw in members:
        sim = _make(grid, kw, 3)
        ws = warmstart.WarmStartSolver(sim, net, judge_sweeps=judge_sweeps)
        recs = []
        for _ in range(steps):
            it, ns = ws.step()
            recs.append((it, ns, ws.last["accepted"]))
        alone.append((recs, {n: sim.download(n) for n in ("u", "v", "p")}))
        sim.close()
    sims = [_make(grid, kw, 3) for grid, kw in members]
    with Batch(sims) as batch:
        bws = warmstart.BatchWarmStart(batch, net, judge_sweeps=judge_sweeps)
        for i in range(steps):
            rec = bws.step()
            for k in range(len(sims)):
                it, ns, acc = alone[k][0][i]
                assert rec[k]["sor_iterations"] == it, (k, i)
                assert rec[k]["norm_squared"] == ns, (k, i)
                assert bws.last["accepted"][k] == acc, (k, i)
    if judge_sweeps < 0:
        assert all(a for recs, _ in alone for (_, _, a) in recs)
    for k, sim in enumerate(sims):
        for n in ("u", "v", "p"):
            np.testing.assert_array_equal(sim.download(n), alone[k][1][n], err_msg=n)
        sim.close()
