"""JSON ingest/egress in the reference's serde layout, its float parsing, and
the NaSt2D .out reader — checked against the reference's fixtures and
snapshots (tests/golden) without a GPU; the GPU round trips are marked gpu."""
import base64
import json

import numpy as np
import pytest

from oracle import oracle as orc
from stroemung_gb300 import jsonio, nast2d, presets
from tests.helpers import assert_bits_equal


def test_serde_float_parse_reproduces_the_reference_snapshot(golden):
    text = golden["fixture_text"]["small_grid_with_boundaries.json"]
    g = jsonio.load_grid(text)  # serde_json's parsing
    snap = golden["snapshots"]["grid_deserialize_boundaries"]
    assert_bits_equal(g["p"].ravel(), np.array(snap["p"]), "pressure as the reference parsed it")
    assert_bits_equal(g["u"].ravel(), np.array(snap["u"]), "u")
    exact = jsonio.load_grid(text, float_parser="exact")
    assert not np.array_equal(exact["p"], g["p"])  # the one value serde rounds differently


def test_serde_float_parser_known_cases():
    # exact cases agree with correct rounding; long significands drop digits
    for s in ("0.0", "-0.0", "1.0", "0.5", "100.0", "1e3", "2.5E-3", "0.2539669433626628"):
        assert jsonio.serde_f64(s) == float(s)
    assert str(jsonio.serde_f64("-0.14603099243353101")) == "-0.146030992433531"
    assert np.signbit(jsonio.serde_f64("-0.0"))


@pytest.mark.parametrize("name", ["small_simulation_with_boundaries.json", "simple_simulation.json"])
def test_loaded_fixture_gives_the_reference_initial_norm(golden, name):
    """With serde's parsing the construction norm is bit-identical to the
    reference's deserialize snapshot (899.9547140394143 for the 4x3 grid)."""
    d = jsonio.simulation_from_json(jsonio.loads(golden["fixture_text"][name]))
    g = d["grid"]
    o = orc.OracleSim(kind=g["kind"], wall_uv=g["wall_uv"], u=g["u"], v=g["v"], p=g["p"],
                      dx=d["cell_size"][0], dy=d["cell_size"][1], delt=d["delt"],
                      gamma=d["gamma"], reynolds=d["reynolds"], eps=d["sor_absolute_epsilon"],
                      omega=d["omega"], max_iterations=d["max_iterations"],
                      iterations=d["iterations"], time=d["time"])
    key = {"small_simulation_with_boundaries.json": "deserialize_small_simulation_with_boundaries",
           "simple_simulation.json": "deserialize_simple_simulation"}[name]
    assert o.state()["initial_norm_squared"] == golden["snapshots"][key]["initial_norm_squared"]


def test_grid_json_round_trip_structure(golden):
    g = jsonio.load_grid(golden["fixture_text"]["small_data.out.json"])
    out = jsonio.grid_to_json((4, 3), g["u"], g["v"], g["p"], g["kind"], g["wall_uv"])
    ref = json.loads(golden["fixture_text"]["small_data.out.json"])
    assert out["cell_type"]["data"] == ref["cell_type"]["data"]
    assert out["size"] == ref["size"]


def test_nast2d_reader_matches_the_reference_converter(golden):
    data = base64.b64decode(golden["nast2d"]["out_b64"])
    raw = nast2d.read_out(data)
    exp = golden["nast2d"]["expected"]
    assert raw["imax"] == exp["imax"] and raw["jmax"] == exp["jmax"]
    for name in ("U", "V", "P", "T"):
        assert_bits_equal(raw[name], np.array(exp[name]), name)
    assert [[int(f) & 16 for f in row] for row in raw["flags"].tolist()] == \
        [[int(f) & 16 for f in row] for row in exp["flags"]]
    grid = nast2d.to_grid(raw)
    rust = golden["nast2d"]["rust_expected"]
    out = jsonio.grid_to_json(rust["size"], grid["u"], grid["v"], grid["p"], grid["kind"],
                              grid["wall_uv"])
    assert out["cell_type"]["data"] == rust["cell_type"]["data"]
    for key, field in (("u", "u"), ("v", "v"), ("pressure", "pressure")):
        assert_bits_equal(np.array(out[key]["data"]), np.array(rust[field]["data"]), key)


def test_oracle_colour_map_basics():
    g = presets.square_obstacle_channel()
    o = orc.OracleSim(kind=g["kind"], wall_uv=g["wall_uv"], u=g["u"], v=g["v"], p=g["p"],
                      dx=0.1, dy=0.1, delt=0.01, gamma=0.9, reynolds=100.0, tau=0.5)
    for _ in range(3):
        o.tick()
    img = o.render(1)
    assert img.shape == (22, 102, 4)
    assert (img[..., 3] == 255).all()
    assert tuple(img[0, 0]) == (127, 127, 127, 255)       # boundary in the speed map
    assert tuple(o.render(0)[0, 0]) == (127, 0, 0, 255)   # boundary in the pressure map
