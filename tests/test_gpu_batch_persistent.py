"""Batches with the persistent solve: the members' pressure solves of a step
run as one cooperative kernel whose CTAs walk the members' tile tables phase
by phase (blocked FP32 sweeps, refinement, FP64 residual, per-member stop
test, the sweep-by-sweep finish), with a grid barrier between phases.

  * every member ends bit-identical to the same simulation stepped alone and
    to the batch's graph loop (members of different sizes and stop rules,
    one of which stops early and takes the sweep-by-sweep finish);
  * the two halves of a step (prepare / solve) give the same fields;
  * a barrier wait that runs out (a limit of one poll) ends the step with
    STRM_ERR_TIMEOUT and no fault; the context stays usable and a batch
    with the default limit then steps correctly.
"""
import numpy as np
import pytest

from stroemung_gb300 import _lib
from stroemung_gb300.batch import Batch
from stroemung_gb300.simulation import StroemungError
from tests.test_gpu_batch import _make, _members

pytestmark = pytest.mark.gpu


def _alone(members, schedule, steps):
    out = []
    for grid, kw in members:
        sim = _make(grid, kw, schedule)
        stats = [sim.run_simulation_tick() for _ in range(steps)]
        out.append((stats, {k: sim.download(k) for k in ("u", "v", "p")}))
        sim.close()
    return out


@pytest.mark.parametrize("schedule", [3, 6])
def test_persistent_batch_matches_single_runs_bitwise(schedule):
    steps = 5
    members = _members()
    alone = _alone(members, schedule, steps)
    sims = [_make(grid, kw, schedule) for grid, kw in members]
    with Batch(sims) as batch:
        batch.set_schedule(schedule)
        batch.set_solver(True)
        st = batch.step(steps)
    for k, sim in enumerate(sims):
        stats, fields = alone[k]
        assert [int(x) for x in st[k]["sor_iterations"]] == [s[0] for s in stats], k
        assert list(st[k]["norm_squared"]) == [s[1] for s in stats], k
        for name in fields:
            np.testing.assert_array_equal(sim.download(name), fields[name],
                                          err_msg=f"member {k} field {name}")
    # the cavity stopped early (its solve finished sweep by sweep), the
    # channels ran to their limits
    assert st[3]["converged"].any() and not st[0]["converged"].any()
    for s in sims:
        s.close()


def test_persistent_halves_match_graph_loop():
    members = _members()[:3]
    a = [_make(g, kw, 3) for g, kw in members]
    b = [_make(g, kw, 3) for g, kw in members]
    with Batch(a) as ba, Batch(b) as bb:
        bb.set_solver(True)
        for _ in range(3):
            ra = ba.step(1)[:, 0]
            bb.prepare()
            rb = bb.solve()
            assert list(ra["sor_iterations"]) == list(rb["sor_iterations"])
            assert list(ra["norm_squared"]) == list(rb["norm_squared"])
    for x, y in zip(a, b):
        for name in ("u", "v", "p"):
            np.testing.assert_array_equal(y.download(name), x.download(name))
        x.close()
        y.close()


def test_persistent_barrier_wait_runs_out_without_fault():
    import torch
    members = _members()[:3]
    sims = [_make(g, kw, 3) for g, kw in members]
    with Batch(sims) as batch:
        batch.set_solver(True, wait_limit=1)
        with pytest.raises(StroemungError) as ei:
            batch.step(1)
        assert ei.value.code == _lib.STRM_ERR_TIMEOUT
    torch.cuda.synchronize()  # the context is intact
    for s in sims:
        s.close()
    # fresh members with the default limit step exactly as alone
    alone = _alone(members, 3, 2)
    sims = [_make(g, kw, 3) for g, kw in members]
    with Batch(sims) as batch:
        batch.set_solver(True)
        batch.step(2)
    for k, sim in enumerate(sims):
        for name, a in alone[k][1].items():
            np.testing.assert_array_equal(sim.download(name), a)
        sim.close()
