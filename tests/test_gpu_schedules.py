"""FP32 sweep schedules of the mixed-precision solve: every temporal-blocking
tile shape gives the per-colour launches' fields bit for bit (graph and
eager execution, inner sweep counts that do not divide evenly into the
blocked launches), and the autotuner picks one of them."""
import numpy as np
import pytest

from stroemung_gb300 import _lib, presets
from stroemung_gb300.simulation import PREC_MIXED, Simulation

EXEC_EAGER = _lib.EXEC_EAGER

pytestmark = pytest.mark.gpu


def _run(grid, schedule, inner, steps=4, execution=0, **kw):
    sim = Simulation(grid=grid, cell_size=(0.01, 0.01), delt=0.005, gamma=0.9, reynolds=300.0,
                     max_iterations=120, tau=0.5, precision=PREC_MIXED, inner_sweeps=inner,
                     sweep_schedule=schedule, execution=execution, **kw)
    stats = [sim.run_simulation_tick() for _ in range(steps)]
    out = {k: sim.download(k) for k in ("u", "v", "p")}
    sim.close()
    return stats, out


def _channel():
    rects = presets.random_rectangles(300, 130, 12, 4, side=(4, 20), x_margin=20)
    return presets.channel(300, 130, rects)


@pytest.mark.parametrize("inner", [16, 7])
def test_blocked_schedules_match_per_colour_bitwise(inner):
    grid = _channel()
    ref_stats, ref = _run(grid, _lib.SWEEPS_PER_COLOUR, inner)
    for v in range(2, _lib.SWEEPS_COUNT):
        stats, got = _run(grid, v, inner)
        assert stats == ref_stats, v
        for k in ref:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"schedule {v} field {k}")


def test_blocked_schedule_eager_matches_graph_and_cavity():
    grid = presets.cavity(96)
    s1, a = _run(grid, 0, 16, steps=3)
    s2, b = _run(grid, 0, 16, steps=3, execution=EXEC_EAGER)
    s3, c = _run(grid, _lib.SWEEPS_PER_COLOUR, 16, steps=3)
    assert s1 == s2 == s3
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
        np.testing.assert_array_equal(a[k], c[k])


def test_autotuner_picks_a_schedule_and_keeps_results():
    grid = _channel()
    sim = Simulation(grid=grid, cell_size=(0.01, 0.01), delt=0.005, gamma=0.9, reynolds=300.0,
                     max_iterations=120, tau=0.5, precision=PREC_MIXED)
    sim.run_simulation_tick()
    best, times = sim.autotune_sweeps(reps=2)
    assert 1 <= best < _lib.SWEEPS_COUNT
    assert all(t > 0 for t in times.values())
    assert times[best] == min(times.values())
    stats = [sim.run_simulation_tick() for _ in range(3)]
    out = {k: sim.download(k) for k in ("u", "v", "p")}
    sim.close()
    ref_stats, ref = _run(grid, _lib.SWEEPS_PER_COLOUR, 16, steps=4)
    assert stats == ref_stats[1:]
    for k in ref:
        np.testing.assert_array_equal(out[k], ref[k])
