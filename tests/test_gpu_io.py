"""GPU-side I/O: JSON load/save in the reference's layout, exact checkpoint
resume, and the headless colour map against the oracle's restatement of
src/visualization.rs."""
import json

import numpy as np
import pytest

from oracle import oracle as orc
from stroemung_gb300 import jsonio, presets
from tests.helpers import assert_bits_equal

pytestmark = pytest.mark.gpu

sim_mod = pytest.importorskip("stroemung_gb300.simulation")
Simulation = sim_mod.Simulation


def _same_json(a, b, path=""):
    if isinstance(a, dict):
        assert set(a) == set(b), path
        for k in a:
            _same_json(a[k], b[k], path + "/" + k)
    elif isinstance(a, list):
        assert len(a) == len(b), path
        for i, (x, y) in enumerate(zip(a, b)):
            _same_json(x, y, f"{path}[{i}]")
    elif isinstance(a, float) or isinstance(b, float):
        x, y = np.float64(a), np.float64(b)
        assert x.view(np.int64) == y.view(np.int64), (path, a, b)
    else:
        assert a == b, path


@pytest.mark.parametrize("name,snap", [
    ("small_simulation_with_boundaries.json", "deserialize_small_simulation_with_boundaries"),
    ("simple_simulation.json", "deserialize_simple_simulation")])
def test_from_json_matches_the_deserialize_snapshot(golden, name, snap):
    """src/simulation.rs:408-420: load, then serialize — the reference's
    snapshot, bit for bit (serde float parsing)."""
    sim = Simulation.from_json(golden["fixture_text"][name])
    got = json.loads(sim.to_json())
    want = golden["snapshots"][snap]
    assert got["initial_norm_squared"] == want["initial_norm_squared"]
    g = got["grid"]
    for key, wkey in (("u", "u"), ("v", "v"), ("pressure", "p")):
        _same_json(g[key]["data"], want["grid"][wkey], key)
    assert g["size"] == want["size"]
    for k in ("cell_size", "delt", "gamma", "reynolds", "sor_absolute_epsilon",
              "max_iterations", "iterations", "time", "omega"):
        _same_json(got[k], want[k], k)


def test_serialize_matches_the_reference_snapshot(golden):
    """src/simulation.rs:422-447 (empty 5x7 grid)."""
    sim = Simulation(grid=presets.empty((5, 7)), cell_size=(1.0, 2.0), delt=1.4, gamma=1.7,
                     reynolds=100.0, sor_absolute_epsilon=0.001, max_iterations=100, omega=1.7)
    got = json.loads(sim.to_json())
    want = golden["snapshots"]["serialize_empty_5x7"]
    assert got["initial_norm_squared"] == want["initial_norm_squared"]
    assert got["grid"]["cell_type"]["data"] == ["Fluid"] * 35
    _same_json(got["grid"]["pressure"]["data"], want["grid"]["p"])


def test_checkpoint_resume_is_exact(tmp_path):
    g = presets.square_obstacle_channel()
    kw = dict(cell_size=(0.1, 0.1), delt=0.01, gamma=0.9, reynolds=100.0, tau=0.5,
              max_iterations=100)
    a = Simulation(grid=g, **kw)
    for _ in range(10):
        a.run_simulation_tick()
    jsonio.save_checkpoint(a, tmp_path / "ck.npz")
    b = jsonio.load_checkpoint(tmp_path / "ck.npz")
    for _ in range(10):
        assert a.run_simulation_tick() == b.run_simulation_tick()
    for n in ("u", "v", "p", "f", "g", "rhs"):
        assert_bits_equal(b.download(n), a.download(n), n)
    assert b.state()["time"] == a.state()["time"]


def test_json_resume_tracks_the_reference_semantics():
    """A JSON save/load is the reference's resume: F/G/RHS recomputed, floats
    re-parsed; continuing from it must match an oracle resumed the same way."""
    g = presets.square_obstacle_channel()
    kw = dict(cell_size=(0.1, 0.1), delt=0.01, gamma=0.9, reynolds=100.0, max_iterations=100)
    a = Simulation(grid=g, sor_order=1, **kw)
    for _ in range(5):
        a.run_simulation_tick()
    text = a.to_json()
    b = Simulation.from_json(text, float_parser="exact", sor_order=1)
    d = jsonio.simulation_from_json(json.loads(text))
    gg = d["grid"]
    o = orc.OracleSim(kind=gg["kind"], wall_uv=gg["wall_uv"], u=gg["u"], v=gg["v"], p=gg["p"],
                      dx=0.1, dy=0.1, delt=d["delt"], gamma=0.9, reynolds=100.0,
                      max_iterations=100, iterations=d["iterations"], time=d["time"],
                      initial_norm_squared=d["initial_norm_squared"])
    for _ in range(5):
        assert b.run_simulation_tick() == o.tick()
    for n in ("u", "v", "p"):
        assert_bits_equal(b.download(n), o.field(n), n)


@pytest.mark.parametrize("color", ["pressure", "speed"])
def test_colour_map_matches_oracle(color, tmp_path):
    rects = presets.random_rectangles(150, 40, 3, 5, x_margin=20)
    g = presets.channel(150, 40, rects)
    kw = dict(dx=0.05, dy=0.05, delt=0.01, gamma=0.9, reynolds=200.0, tau=0.5,
              max_iterations=30)
    o = orc.OracleSim(kind=g["kind"], wall_uv=g["wall_uv"], u=g["u"], v=g["v"], p=g["p"], **kw)
    s = Simulation(grid=g, cell_size=(0.05, 0.05), delt=0.01, gamma=0.9, reynolds=200.0,
                   tau=0.5, max_iterations=30, sor_order=1)
    for _ in range(6):
        assert s.run_simulation_tick() == o.tick()
    ct = {"pressure": 0, "speed": 1}[color]
    img = s.render(color)
    ref = o.render(ct)
    assert img.shape == ref.shape == (42, 152, 4)
    assert np.array_equal(img, ref)
    sim_mod.write_png(tmp_path / f"{color}.png", img)
    assert (tmp_path / f"{color}.png").stat().st_size > 100
