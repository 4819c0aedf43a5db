"""Stop rules and residual histories of the pressure solve: the relative
rule ends each solve at the first norm below eps^2 x the norm it started
from, in FP64 and in mixed precision, in graph and eager execution."""
import numpy as np
import pytest

from stroemung_gb300 import _lib, presets
from stroemung_gb300.simulation import PREC_FP64, PREC_MIXED, Simulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_MIXED])
@pytest.mark.parametrize("execution", [_lib.EXEC_GRAPH, _lib.EXEC_EAGER])
def test_relative_rule_stops_at_first_norm_below_target(precision, execution):
    eps = 1e-3
    sim = Simulation(grid=presets.cavity(64), cell_size=(1 / 64, 1 / 64), delt=1e-3, gamma=0.9,
                     reynolds=100.0, sor_absolute_epsilon=eps, max_iterations=5000, omega=1.8,
                     tau=0.5, precision=precision, strict_eps=_lib.STOP_RELATIVE,
                     execution=execution)
    for _ in range(3):
        it, ns = sim.run_simulation_tick()
        h = sim.residual_history()
        assert h[0, 0] == 0  # the starting norm
        start = h[0, 1]
        assert ns == h[-1, 1] and it == int(h[-1, 0])
        assert ns < eps * eps * start
        # no earlier recorded norm met the target
        assert not (h[1:-1, 1] < eps * eps * start).any()
        assert sim.state()["last_converged"]
    sim.close()


def test_relative_rule_is_refused_for_the_lexicographic_order():
    sim = Simulation(grid=presets.cavity(16), cell_size=(1 / 16, 1 / 16), delt=1e-3, gamma=0.9,
                     reynolds=100.0, max_iterations=10)
    with pytest.raises(Exception):
        sim.set_mode(sor_order=_lib.SOR_LEXICOGRAPHIC, strict_eps=_lib.STOP_RELATIVE)
    sim.close()


@pytest.mark.parametrize("norm_cells", [_lib.NORM_ALL_INTERIOR, _lib.NORM_FLUID,
                                        _lib.NORM_FLUID_MEAN_FREE])
def test_fast_solve_norm_matches_the_fields(norm_cells):
    """FAST FP64 solves sum the black fluid cells' residual inside the black
    pass and the other cells in the residual pass; the norm they report
    equals the norm of the fields they leave (every residual kind)."""
    from stroemung_gb300.simulation import ARITH_FAST
    g = presets.channel(96, 40, [(30, 12, 8, 6), (60, 20, 5, 9)])
    sim = Simulation(grid=g, cell_size=(0.01, 0.01), delt=0.002, gamma=0.9, reynolds=200.0,
                     max_iterations=37, tau=0.5, arithmetic=ARITH_FAST,
                     norm_cells=norm_cells, strict_eps=_lib.STOP_STRICT,
                     sor_absolute_epsilon=1e-12)
    for _ in range(3):
        it, ns = sim.run_simulation_tick()
    # the last solve's fields: p before the velocity update is what the norm saw
    p, rhs = sim.download("p"), sim.download("rhs")
    dx2 = 0.01 * 0.01
    r = (p[2:, 1:-1] + p[:-2, 1:-1]) / dx2 + (p[1:-1, 2:] + p[1:-1, :-2]) / dx2 \
        - 2 * (2 / dx2) * p[1:-1, 1:-1] - rhs[1:-1, 1:-1]
    fluid = sim._kind[1:-1, 1:-1] == 0
    nf = float(sim.state()["fluid_cells"])
    if norm_cells == _lib.NORM_ALL_INTERIOR:
        want = (r ** 2).sum() / nf
    elif norm_cells == _lib.NORM_FLUID:
        want = (r[fluid] ** 2).sum() / nf
    else:
        rf = r[fluid]
        want = ((rf ** 2).sum() - rf.sum() ** 2 / nf) / nf
    assert it == 37
    np.testing.assert_allclose(ns, want, rtol=1e-8)
    sim.close()


@pytest.mark.parametrize("norm_cells", [_lib.NORM_ALL_INTERIOR, _lib.NORM_FLUID,
                                        _lib.NORM_FLUID_MEAN_FREE])
@pytest.mark.parametrize("execution", [_lib.EXEC_GRAPH, _lib.EXEC_EAGER])
def test_fast_solve_matches_exact_with_early_stops(norm_cells, execution):
    """FAST arithmetic against EXACT on a cavity with an obstacle under the
    relative rule, where solves stop early (the FAST solve then rolls back
    the next iteration's red pass and boundary copy): the same iteration
    counts, norms and fields within 1e-9, for every residual kind."""
    from stroemung_gb300.simulation import ARITH_EXACT, ARITH_FAST
    g = presets.cavity(40)
    g["kind"][15:20, 14:22] = presets.NO_SLIP
    prm = dict(grid=g, cell_size=(1 / 40, 1 / 40), delt=2e-3, gamma=0.9, reynolds=100.0,
               sor_absolute_epsilon=0.3, max_iterations=3000, omega=1.7, tau=0.5,
               strict_eps=_lib.STOP_RELATIVE, norm_cells=norm_cells)
    fast = Simulation(arithmetic=ARITH_FAST, execution=execution, **prm)
    exact = Simulation(arithmetic=ARITH_EXACT, **prm)
    iters = []
    for step in range(6):
        i_f, n_f = fast.run_simulation_tick()
        i_e, n_e = exact.run_simulation_tick()
        assert i_f == i_e, (step, i_f, i_e)
        assert abs(n_f - n_e) <= 1e-9 * abs(n_e), (step, n_f, n_e)
        iters.append(i_f)
    # the fluid norms stop every solve early; the norm over every interior
    # cell keeps the obstacle's stale boundary residual and stops the first
    assert min(iters) < prm["max_iterations"], iters
    if norm_cells != _lib.NORM_ALL_INTERIOR:
        assert max(iters) < prm["max_iterations"], iters
    for n in ("u", "v", "p"):
        a, b = fast.download(n), exact.download(n)
        assert np.linalg.norm(a - b) <= 1e-9 * np.linalg.norm(b), n
    fast.close()
    exact.close()
