"""The FAST arithmetic's pointwise kernels against the oracle, phase by phase.

In FAST mode F, G and RHS come from the face-flux stencil (fused
multiply-adds, reciprocal multiplies; src/simulation.rs:122-214 and
src/math.rs:19-174 regrouped) and the velocity update from fused
multiply-adds (src/simulation.rs:287-322).  Starting from the same fields
as the oracle, on random layouts with every boundary kind and on an
all-fluid grid (whose ring cells keep their old F and G):

  * F, G, RHS and the updated u, v within 1e-12 relative L2 of the oracle —
    the bound for the pointwise kernels;
  * boundary copies exact: F = u and G = v wherever the reference copies;
  * the speed range within 1e-12 relative.
"""
import numpy as np
import pytest

from oracle import oracle as orc
from stroemung_gb300 import presets
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

sim_mod = pytest.importorskip("stroemung_gb300.simulation")

PRM = dict(cell_size=(0.1, 0.07), delt=0.002, gamma=0.8, reynolds=50.0)


def _layouts():
    from tests.test_host_boundary import random_layout
    out = []
    for seed in range(6):
        rng = np.random.default_rng(300 + seed)
        nx, ny = int(rng.integers(20, 90)), int(rng.integers(12, 70))
        for _ in range(100):
            kind = random_layout(rng, nx, ny, int(rng.integers(0, 8)))
            if orc.classify(kind)[2] is None:
                break
        else:
            continue
        out.append((f"random{seed}", kind, rng))
    rng = np.random.default_rng(399)
    out.append(("all_fluid", np.zeros((70, 45), np.uint8), rng))
    return out


@pytest.mark.parametrize("name,kind,rng", _layouts(), ids=lambda x: x if isinstance(x, str) else "")
def test_fast_pointwise_phases_match_oracle(name, kind, rng):
    from stroemung_gb300.simulation import ARITH_FAST, Simulation
    nx, ny = kind.shape
    g = presets.empty((nx, ny))
    g["kind"] = kind
    g["wall_uv"] = rng.normal(size=(nx, ny, 2))
    for n in ("u", "v", "p"):
        g[n] = rng.normal(size=(nx, ny))
    o = orc.OracleSim(kind=kind, wall_uv=g["wall_uv"], u=g["u"], v=g["v"], p=g["p"],
                      dx=PRM["cell_size"][0], dy=PRM["cell_size"][1], delt=PRM["delt"],
                      gamma=PRM["gamma"], reynolds=PRM["reynolds"])
    with Simulation(grid=g, arithmetic=ARITH_FAST, **PRM) as s:
        # the same F, G, RHS to start from (construction computes them)
        for n in ("f", "g", "rhs"):
            s.upload(n, o.field(n))
        o.set_boundary_u_and_v()
        s.set_boundary_u_and_v()
        u, v = o.field("u"), o.field("v")
        assert np.array_equal(s.download("u"), u) and np.array_equal(s.download("v"), v)
        o.calculate_f_and_g()
        o.calculate_rhs()
        s.calculate_f_g_rhs()
        for n in ("f", "g", "rhs"):
            err = rel_l2(s.download(n), o.field(n))
            assert err <= 1e-12, (name, n, err)
        bnd = kind != 0
        keep_f = bnd.copy()
        keep_f[:-1] |= bnd[1:]
        keep_g = bnd.copy()
        keep_g[:, :-1] |= bnd[:, 1:]
        assert np.array_equal(s.download("f")[keep_f], u[keep_f]), name
        assert np.array_equal(s.download("g")[keep_g], v[keep_g]), name
        o.copy_pressure_to_boundaries()
        s.copy_pressure_to_boundaries()
        o.set_u_and_v()
        s.set_u_and_v()
        for n in ("u", "v"):
            err = rel_l2(s.download(n), o.field(n))
            assert err <= 1e-12, (name, n, err)
        sr_s, sr_o = s.state()["speed_range"], o.state()["speed_range"]
        for a, b in zip(sr_s, sr_o):
            assert abs(a - b) <= 1e-12 * abs(b), (name, sr_s, sr_o)
