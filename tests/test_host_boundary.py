"""Host half of the device path, checked against the oracle without a GPU:
the cell classification and the compiled (gather/scatter) boundary program
must reproduce the reference's sequential boundary pass and its restore list
bit for bit, on the reference's fixtures and on random layouts with every
boundary kind."""
import numpy as np
import pytest

from oracle import oracle as orc
from stroemung_gb300 import presets
from stroemung_gb300.simulation import BoundaryTooThinError, host_boundary_pass, host_classify
from tests.helpers import assert_bits_equal


def random_layout(rng, nx, ny, nblocks):
    kind = np.zeros((nx, ny), np.uint8)
    kind[:, 0] = rng.integers(1, 5)
    kind[:, ny - 1] = rng.integers(1, 5)
    kind[0, :] = rng.integers(1, 5)
    kind[nx - 1, :] = rng.integers(1, 5)
    # random ring kinds cell by cell
    ring = np.zeros((nx, ny), bool)
    ring[[0, nx - 1], :] = True
    ring[:, [0, ny - 1]] = True
    kind[ring] = rng.integers(1, 5, size=ring.sum())
    for _ in range(nblocks):
        w, h = rng.integers(2, 5, size=2)
        x0 = rng.integers(1, max(2, nx - w))
        y0 = rng.integers(1, max(2, ny - h))
        kind[x0:x0 + w, y0:y0 + h] = rng.integers(1, 5)
    return kind


def oracle_boundary(kind, wall, u, v):
    """Oracle: sequential pass, then the restore replay observed through
    set_u_and_v with F = G = 0, p = 0 on every cell."""
    nx, ny = kind.shape
    sim = orc.OracleSim(kind=kind, wall_uv=wall, u=u, v=v, p=np.zeros_like(u), dx=0.1,
                        dy=0.1, delt=0.01, gamma=0.9, reynolds=100.0)
    sim.set_field("u", u)
    sim.set_field("v", v)
    sim.set_boundary_u_and_v()
    u1, v1 = sim.field("u"), sim.field("v")
    sim.set_field("f", np.zeros_like(u))
    sim.set_field("g", np.zeros_like(u))
    sim.set_field("p", np.zeros_like(u))
    sim.set_u_and_v()
    return u1, v1, sim.field("u"), sim.field("v")


def check_layout(kind, wall, u, v):
    u1, v1, ur, vr = oracle_boundary(kind, wall, u, v)
    hu, hv, hru, hrv = host_boundary_pass(kind, wall, u, v)
    assert_bits_equal(hu, u1, "u after the boundary pass")
    assert_bits_equal(hv, v1, "v after the boundary pass")
    edges, _ = host_classify(kind)
    sel = (kind != 0) & (edges != 0)
    assert_bits_equal(hru[sel], ur[sel], "restore u")
    assert_bits_equal(hrv[sel], vr[sel], "restore v")


def test_classification_matches_oracle_on_fixtures(golden):
    for name in ("small_grid_with_boundaries.json", "small_data.out.json"):
        g = golden["fixtures"][name]
        kind = np.array(g["kind"], np.uint8).reshape(g["size"])
        e_host, fc = host_classify(kind)
        e_orc, fc_orc, bad = orc.classify(kind)
        assert bad is None
        assert np.array_equal(e_host, e_orc) and fc == fc_orc


def test_thin_wall_reported_like_the_reference(golden):
    nx, ny = golden["thin_boundary"]["size"]
    for cells in golden["thin_boundary"]["examples"]:
        kind = np.zeros((nx, ny), np.uint8)
        for x, y in cells:
            kind[x, y] = 1
        with pytest.raises(BoundaryTooThinError):
            host_classify(kind)


def test_boundary_pass_on_the_tick_fixture():
    g = presets.simple_inflow((4, 3))
    rng = np.random.default_rng(1)
    check_layout(g["kind"], g["wall_uv"], rng.normal(size=(4, 3)), rng.normal(size=(4, 3)))


@pytest.mark.parametrize("seed", range(40))
def test_boundary_pass_random_layouts(seed):
    rng = np.random.default_rng(seed)
    nx, ny = int(rng.integers(4, 14)), int(rng.integers(4, 14))
    for _ in range(50):
        kind = random_layout(rng, nx, ny, int(rng.integers(0, 5)))
        _, _, bad = orc.classify(kind)
        if bad is None:
            break
    else:
        pytest.skip("no valid layout drawn")
    wall = rng.normal(size=(nx, ny, 2))
    # some exact zeros so that the sign of zero is exercised
    u = np.where(rng.random((nx, ny)) < 0.2, 0.0, rng.normal(size=(nx, ny)))
    v = np.where(rng.random((nx, ny)) < 0.2, -0.0, rng.normal(size=(nx, ny)))
    check_layout(kind, wall, u, v)


def test_channel_layouts():
    for seed in range(3):
        rects = presets.random_rectangles(200, 60, 6, seed, x_margin=10)
        g = presets.channel(200, 60, rects)
        rng = np.random.default_rng(seed)
        check_layout(g["kind"], g["wall_uv"], g["u"] + rng.normal(size=g["u"].shape) * 0.1,
                     rng.normal(size=g["u"].shape) * 0.1)
    g = presets.cavity(30)
    rng = np.random.default_rng(7)
    check_layout(g["kind"], g["wall_uv"], rng.normal(size=g["u"].shape),
                 rng.normal(size=g["u"].shape))
