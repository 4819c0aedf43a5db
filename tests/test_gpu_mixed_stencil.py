"""The FP32 F/G/RHS stencil of mixed precision against the FP64 path on the
same state: boundary values are exact copies, and the interior increments
F - u, G - v and the RHS are within FP32 rounding of the increment (the
stencil keeps u and v as hi/lo float pairs, so no operation cancels u)."""
import numpy as np
import pytest

from stroemung_gb300 import presets
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu


def test_fp32_stencil_matches_fp64_on_the_same_state():
    from stroemung_gb300.simulation import ARITH_FAST, PREC_MIXED, Simulation
    rects = presets.random_rectangles(160, 64, 4, 3, x_margin=16)
    g = presets.channel(160, 64, rects)
    prm = dict(cell_size=(0.02, 0.02), delt=0.01, gamma=0.9, reynolds=300.0,
               sor_absolute_epsilon=1e-3, max_iterations=200, omega=1.7, tau=0.5,
               arithmetic=ARITH_FAST)
    warm = Simulation(grid=g, **prm)
    for _ in range(12):
        warm.run_simulation_tick()
    state = dict(g, u=warm.download("u"), v=warm.download("v"), p=warm.download("p"))
    warm.close()
    a = Simulation(grid=state, **prm)
    b = Simulation(grid=state, precision=PREC_MIXED, **prm)
    a.tick_prepare()
    b.tick_prepare()
    u, v = state["u"], state["v"]
    fa, fb = a.download("f"), b.download("f")
    ga, gb = a.download("g"), b.download("g")
    ra, rb = a.download("rhs"), b.download("rhs")
    fluid = g["kind"] == 0
    # non-fluid cells: F = u, G = v copied exactly, as in the FP64 path
    np.testing.assert_array_equal(fb[~fluid], fa[~fluid])
    np.testing.assert_array_equal(gb[~fluid], ga[~fluid])
    inner = np.zeros_like(fluid)
    inner[1:-1, 1:-1] = fluid[1:-1, 1:-1]
    inc_f, inc_g = (fa - u)[inner], (ga - v)[inner]
    assert np.abs(inc_f).max() > 0 and np.abs(inc_g).max() > 0
    assert rel_l2((fb - u)[inner], inc_f) < 1e-6, rel_l2((fb - u)[inner], inc_f)
    assert rel_l2((gb - v)[inner], inc_g) < 1e-6, rel_l2((gb - v)[inner], inc_g)
    assert rel_l2(rb[1:, 1:], ra[1:, 1:]) < 1e-6, rel_l2(rb[1:, 1:], ra[1:, 1:])
    a.close()
    b.close()
