"""Regenerates tests/golden/reference_golden.json from the reference's own tests.

Run it with the reference's source tree given as the first argument or in
the STROEMUNG_REF environment variable:

    python tests/golden/make_golden.py <path to the stroemung checkout>

It reads, as text, the known-answer tables of src/math.rs:192-402 and
src/simulation.rs:449-569, the classification tables of
src/grid/mod.rs:683-801, the insta snapshots under src/snapshots,
src/grid/snapshots and tests/snapshots, the JSON fixtures under src/test_data
and tests/test_data, and the asserted tick results of
src/simulation.rs:597-606.  Nothing here is computed: every number is the
reference's.  The test suite reads only the JSON this script writes.
"""
from __future__ import annotations

import ast
import json
import os
import re
import sys
from pathlib import Path

REF: Path = Path()  # the reference checkout, set by main()
OUT = Path(__file__).resolve().parent / "reference_golden.json"


def _strip_comments(src: str) -> str:
    return re.sub(r"//[^\n]*", "", src)


def _fn_body(src: str, name: str) -> str:
    m = re.search(r"fn\s+" + re.escape(name) + r"\s*\(", src)
    if not m:
        raise KeyError(name)
    i = src.index("{", m.end())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[i + 1:j]
    raise ValueError(name)


def _test_cases(src: str, fn: str):
    """Parses `let test_cases = [ (...), ... ];` of a Rust test into Python."""
    body = _strip_comments(_fn_body(src, fn))
    m = re.search(r"let\s+test_cases\s*=\s*\[", body)
    start = m.end() - 1
    depth = 0
    for j in range(start, len(body)):
        if body[j] == "[":
            depth += 1
        elif body[j] == "]":
            depth -= 1
            if depth == 0:
                lit = body[start:j + 1]
                break
    lit = lit.replace("array![", "[")
    return [list(t) for t in ast.literal_eval(lit)]


def _snapshot_json(path: Path):
    text = path.read_text()
    return json.loads(text.split("---", 2)[2])


def _snapshot_text(path: Path) -> str:
    return path.read_text().split("---", 2)[2].strip("\n")


def _cells(cell_json):
    """ndarray JSON of Cell -> (kind codes, inflow velocities) row-major."""
    kinds, wall = [], []
    for c in cell_json["data"]:
        if c == "Fluid":
            kinds.append(0)
            wall.append([0.0, 0.0])
        elif c["Boundary"] == "NoSlip":
            kinds.append(1)
            wall.append([0.0, 0.0])
        elif c["Boundary"] == "Outflow":
            kinds.append(2)
            wall.append([0.0, 0.0])
        else:
            kinds.append(3)
            wall.append(list(c["Boundary"]["Inflow"]["velocity"]))
    return kinds, wall


def _grid_json(g):
    kinds, wall = _cells(g["cell_type"])
    return {"size": g["size"], "kind": kinds, "wall_uv": wall, "u": g["u"]["data"],
            "v": g["v"]["data"], "p": g["pressure"]["data"]}


def _sim_json(s):
    out = {k: s[k] for k in ("size", "cell_size", "delt", "gamma", "reynolds",
                             "sor_absolute_epsilon", "max_iterations", "iterations", "time",
                             "omega")}
    out["initial_norm_squared"] = s.get("initial_norm_squared")
    out["grid"] = _grid_json(s["grid"])
    return out


EDGE_CODES = {"North": 1, "NorthEast": 2, "East": 3, "SouthEast": 4, "South": 5,
              "SouthWest": 6, "West": 7, "NorthWest": 8}


def _edge_list(text: str):
    return [0 if g == "None" else EDGE_CODES[g2]
            for g, g2 in re.findall(r"(None|Some\(EdgeType::(\w+))", text)]


def main():
    global REF
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("STROEMUNG_REF", "")
    if not root:
        sys.exit("usage: make_golden.py <stroemung checkout>  (or set STROEMUNG_REF)")
    REF = Path(root)
    # only the #[cfg(test)] modules hold the tables
    math_rs = (REF / "src/math.rs").read_text().split("#[cfg(test)]", 1)[1]
    sim_rs = (REF / "src/simulation.rs").read_text().split("#[cfg(test)]", 1)[1]
    grid_rs = (REF / "src/grid/mod.rs").read_text().split("#[cfg(test)]", 1)[1]
    snaps = REF / "src/snapshots"
    gold = {"source": "wickedchicken/stroemung tests and snapshots"}

    gold["math"] = {
        "du2dx": _test_cases(math_rs, "test_du2dx"),
        "duvdx": _test_cases(math_rs, "test_duvdx"),
        "duvdy": _test_cases(math_rs, "test_duvdy"),
        "dv2dy": _test_cases(math_rs, "test_dv2dy"),
        "laplacian": _test_cases(math_rs, "test_lapacian"),
    }
    gold["calculate_f"] = _test_cases(sim_rs, "test_calculate_f")
    gold["calculate_g"] = _test_cases(sim_rs, "test_calculate_g")

    # src/grid/mod.rs:683-705 thin_boundary
    body = _strip_comments(_fn_body(grid_rs, "thin_boundary"))
    vecs = re.search(r"vec!\[(vec!\[.*?\]),\s*(vec!\[.*?\])\]", body, re.S)
    thin = []
    for v in vecs.groups():
        thin.append([list(t) for t in ast.literal_eval(v.replace("vec!", ""))])
    gold["thin_boundary"] = {"size": [3, 3], "examples": thin}

    # src/grid/mod.rs:707-801 rebuild_boundary_list
    body = _strip_comments(_fn_body(grid_rs, "rebuild_boundary_list"))
    ex_src = body[body.index("let examples"):body.index("for (expected_boundaries")]
    parts = re.split(r"\(\s*vec!\[", ex_src)[1:]
    examples = []
    for part in parts:
        idx_txt, rest = part.split("]", 1)
        cells = [list(t) for t in ast.literal_eval("[" + idx_txt + "]")]
        examples.append({"boundaries": cells, "edges": _edge_list(rest)})
    gold["rebuild_boundary_list"] = {"size": [3, 3], "examples": examples}

    # JSON fixtures and their snapshots
    gold["fixtures"] = {}
    for name in ("simple_grid.json", "small_grid_with_boundaries.json"):
        gold["fixtures"][name] = _grid_json(json.loads((REF / "src/test_data" / name).read_text()))
    for name in ("simple_simulation.json", "small_simulation_with_boundaries.json"):
        gold["fixtures"][name] = _sim_json(json.loads((REF / "src/test_data" / name).read_text()))
    gold["fixtures"]["small_data.out.json"] = _grid_json(
        json.loads((REF / "tests/test_data/small_data.out.json").read_text()))

    gold["snapshots"] = {
        "deserialize_simple_simulation": _sim_json(
            _snapshot_json(snaps / "stroemung__simulation__tests__deserialize.snap")),
        "deserialize_small_simulation_with_boundaries": _sim_json(
            _snapshot_json(snaps / "stroemung__simulation__tests__deserialize-2.snap")),
        "serialize_empty_5x7": _sim_json(
            _snapshot_json(snaps / "stroemung__simulation__tests__serialize.snap")),
        "grid_deserialize_boundaries": _grid_json(_snapshot_json(
            REF / "src/grid/snapshots/stroemung__grid__tests__deserialize_boundaries.snap")),
        "grid_deserialize_boundaries_list": _snapshot_text(
            REF / "src/grid/snapshots/stroemung__grid__tests__deserialize_boundaries-2.snap"),
        "file_parsing_deserialize": _grid_json(_snapshot_json(
            REF / "tests/snapshots/test_file_parsing__deserialize.snap")),
    }
    bl = gold["snapshots"]["grid_deserialize_boundaries_list"]
    sorted_part = bl.split("Sorted Boundary List:")[1]
    gold["snapshots"]["grid_deserialize_boundaries_edges"] = [
        {"cell": [int(a), int(b)], "edge": 0 if name == "" else EDGE_CODES[name]}
        for a, b, name in re.findall(r"\(\((\d+), (\d+)\), (?:None|Some\((\w+))", sorted_part)
    ]

    # src/simulation.rs:571-618 simulation_tick on presets::simple_inflow([4, 3])
    tick = {}
    names = ["f", "g", "rhs", "sim"]
    for k, suffix in enumerate(["", "-2", "-3", "-4"]):
        tick["tick1_" + names[k]] = _snapshot_json(
            snaps / f"stroemung__simulation__tests__simulation_tick{suffix}.snap")
    for k, suffix in enumerate(["-5", "-6", "-7", "-8"]):
        tick["tick101_" + names[k]] = _snapshot_json(
            snaps / f"stroemung__simulation__tests__simulation_tick{suffix}.snap")
    tick["tick201_sim"] = _snapshot_json(
        snaps / "stroemung__simulation__tests__simulation_tick-9.snap")
    for k in list(tick):
        if k.endswith("_sim"):
            tick[k] = _sim_json(tick[k])
        else:
            tick[k] = tick[k]["data"]
    body = _fn_body(sim_rs, "simulation_tick")
    iters = re.findall(r"assert_eq!\((?:last_)?sor_iterations,\s*(\d+)\)", body)
    norms = re.findall(r"assert_eq!\((?:last_)?norm_squared,\s*([-0-9.e]+)\)", body)
    tick["tick1_result"] = [int(iters[0]), float(norms[0])]
    tick["tick101_result"] = [int(iters[1]), float(norms[1])]
    params = {}
    for key in ("cell_size", "delt", "gamma", "reynolds", "sor_absolute_epsilon",
                "max_iterations", "omega"):
        m = re.search(key + r":\s*(\[[^\]]*\]|[^,\n]+),", body)
        params[key] = ast.literal_eval(m.group(1).strip())
    params["size"] = [4, 3]
    tick["params"] = params
    gold["simulation_tick"] = tick

    # python/test_generate_test_data.py: a 440-byte NaSt2D .out file and the
    # grid JSON the reference's converter makes of it
    import base64
    td = REF / "python" / "test_data"
    gold["nast2d"] = {
        "out_b64": base64.b64encode((td / "small_data.out").read_bytes()).decode(),
        "expected": json.loads((td / "small_data.out_expected.json").read_text()),
        "rust_expected": json.loads((td / "small_data.out_rust_expected.json").read_text()),
    }
    # the grid/simulation JSON fixtures as text, so that loaders can be checked
    # with the reference's own float parsing
    gold["fixture_text"] = {
        name: (REF / "src" / "test_data" / name).read_text()
        for name in ("simple_grid.json", "small_grid_with_boundaries.json",
                     "simple_simulation.json", "small_simulation_with_boundaries.json")
    }
    gold["fixture_text"]["small_data.out.json"] = (
        REF / "tests" / "test_data" / "small_data.out.json").read_text()

    OUT.write_text(json.dumps(gold, indent=1, sort_keys=True) + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
