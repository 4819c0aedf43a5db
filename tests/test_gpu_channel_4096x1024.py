"""GPU parity on the benchmarked workload itself: the 4096 x 1024 channel with
64 seeded rectangles (Re 400, tau 0.5, gamma 0.9, omega 1.7, eps 1e-3).

The reference's tick (src/simulation.rs:324-333) with its pressure solve
(src/simulation.rs:239-285) runs on the oracle in red-black order and on the
GPU through the C ABI, two steps each with the solve capped at 20
iterations (an uncapped step would keep the oracle busy for minutes).  At
this size the GPU runs partial tiles at the 4098 x 1026 edges, 608 residual
blocks, the boundary-cell list of 64 obstacles and the compiled boundary
program of the whole channel; small grids exercise none of these at scale.

Bars:
  * EXACT arithmetic: F, G, RHS, u, v, p bit-identical to the oracle after
    each step, equal iteration counts, norms within 1e-12 relative (only the
    residual sum's order differs), equal time step;
  * FAST arithmetic (fused multiply-adds, reciprocal multiplies, the face-flux
    F/G stencil): F, G and RHS of the first step, computed from the same
    u and v as the oracle's, within 1e-12 relative L2 (the bound for the
    pointwise kernels); after the solves every field within 1e-9 relative
    L2, equal iteration counts, norms within 1e-9.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from stroemung_gb300 import presets
from tests.helpers import assert_bits_equal, rel_l2

pytestmark = pytest.mark.gpu

IMAX, JMAX, NRECTS, SEED = 4096, 1024, 64, 0
PRM = dict(dx=0.01, dy=0.01, delt=0.005, gamma=0.9, reynolds=400.0, eps=1e-3, omega=1.7,
           max_iterations=20, tau=0.5)
STEPS = 2


@pytest.fixture(scope="module")
def oracle_run():
    """The oracle's red-black run: per step (iterations, norm, delt, fields)."""
    orc.build()
    rects = presets.random_rectangles(IMAX, JMAX, NRECTS, SEED)
    g = presets.channel(IMAX, JMAX, rects)
    o = orc.OracleSim(kind=g["kind"], wall_uv=g["wall_uv"], u=g["u"], v=g["v"], p=g["p"],
                      sor_order=orc.RED_BLACK, **PRM)
    steps = []
    for _ in range(STEPS):
        it, ns = o.tick()
        steps.append({"it": it, "ns": ns, "delt": o.state()["delt"],
                      "fields": {n: o.field(n) for n in ("u", "v", "p", "f", "g", "rhs")}})
    return g, steps


def _gpu(g, arithmetic):
    from stroemung_gb300.simulation import Simulation
    return Simulation(grid=g, cell_size=(PRM["dx"], PRM["dy"]), delt=PRM["delt"],
                      gamma=PRM["gamma"], reynolds=PRM["reynolds"],
                      sor_absolute_epsilon=PRM["eps"], max_iterations=PRM["max_iterations"],
                      omega=PRM["omega"], tau=PRM["tau"], sor_order=0, arithmetic=arithmetic)


def test_exact_red_black_bit_identical_to_oracle(oracle_run):
    from stroemung_gb300.simulation import ARITH_EXACT
    g, steps = oracle_run
    with _gpu(g, ARITH_EXACT) as s:
        for k, ref in enumerate(steps):
            it, ns = s.run_simulation_tick()
            assert it == ref["it"], (k, it, ref["it"])
            assert abs(ns - ref["ns"]) <= 1e-12 * abs(ref["ns"]), (k, ns, ref["ns"])
            assert s.state()["delt"] == ref["delt"], k
            for n, a in ref["fields"].items():
                assert_bits_equal(s.download(n), a, f"step {k} {n}")


def test_fast_red_black_within_1e9_of_oracle(oracle_run):
    from stroemung_gb300.simulation import ARITH_FAST
    g, steps = oracle_run
    with _gpu(g, ARITH_FAST) as s:
        for k, ref in enumerate(steps):
            it, ns = s.run_simulation_tick()
            assert it == ref["it"], (k, it, ref["it"])
            assert abs(ns - ref["ns"]) <= 1e-9 * abs(ref["ns"]), (k, ns, ref["ns"])
            for n, a in ref["fields"].items():
                err = rel_l2(s.download(n), a)
                bound = 1e-12 if k == 0 and n in ("f", "g", "rhs") else 1e-9
                assert err <= bound, (k, n, err)
