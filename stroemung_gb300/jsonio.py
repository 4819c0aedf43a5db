"""JSON ingest / egress and checkpoints in the reference's serde layout.

The reference saves and loads whole simulations with serde_json
(src/simulation.rs:30-120, src/grid/mod.rs:85-153, 334-341):

    {"size": [nx, ny], "cell_size": [dx, dy], "delt", "gamma", "reynolds",
     "initial_norm_squared" (optional), "sor_absolute_epsilon", "max_iterations",
     "iterations", "time", "omega",
     "grid": {"size", "pressure", "u", "v", "cell_type"}}

with every field an ndarray ``{"v": 1, "dim": [nx, ny], "data": [...]}`` in
row-major order (y fastest) and cells as ``"Fluid"``,
``{"Boundary": "NoSlip"}``, ``{"Boundary": "Outflow"}`` or
``{"Boundary": {"Inflow": {"velocity": [u, v]}}}``; F, G and RHS are not
saved (they are recomputed on load).

Numbers are read, by default, the way serde_json 1.0.140 (the version in the
reference's Cargo.lock, default features, i.e. without ``float_roundtrip``)
reads them: the decimal digits are accumulated into a u64 significand (digits
that would overflow it are dropped), the significand is converted to f64 and
then multiplied or divided once by the correctly rounded power of ten.  That
is not always correctly rounded, and reproducing it is what makes a loaded
fixture bit-identical to the reference's (its deserialize snapshot holds
-0.146030992433531 for the text -0.14603099243353101).  ``float_parser="exact"``
uses Python's correctly rounded reader instead.

``save_checkpoint`` / ``load_checkpoint`` write every field, F, G and RHS
included, in binary (numpy .npz) for an exact resume.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

from . import presets

_POW10 = [float("1e%d" % i) for i in range(309)]
_U64_MAX = 2 ** 64 - 1


def serde_f64(text: str) -> float:
    """serde_json's default f64 parse (the non-float_roundtrip path)."""
    s = text
    negative = s.startswith("-")
    if negative:
        s = s[1:]
    exp = 0
    for marker in ("e", "E"):
        if marker in s:
            s, e = s.split(marker, 1)
            exp = int(e)
            break
    int_part, _, frac_part = s.partition(".")
    significand = 0
    exponent = 0
    overflowed = False
    for ch in int_part:
        d = ord(ch) - 48
        if not overflowed and (significand > _U64_MAX // 10 or
                               (significand == _U64_MAX // 10 and d > _U64_MAX % 10)):
            overflowed = True
        if overflowed:
            exponent += 1  # a digit dropped before the point still scales
            continue
        significand = significand * 10 + d
    for ch in frac_part:
        d = ord(ch) - 48
        if not overflowed and (significand > _U64_MAX // 10 or
                               (significand == _U64_MAX // 10 and d > _U64_MAX % 10)):
            overflowed = True
        if overflowed:
            continue
        significand = significand * 10 + d
        exponent -= 1
    exponent += exp
    f = float(significand)
    while True:
        if abs(exponent) < len(_POW10):
            f = f * _POW10[exponent] if exponent >= 0 else f / _POW10[-exponent]
            break
        if f == 0.0:
            break
        if exponent >= 0:
            raise ValueError(f"number out of range: {text}")
        f /= 1e308
        exponent += 308
    return -f if negative else f


def loads(text: str, float_parser: str = "serde"):
    if float_parser == "serde":
        return json.loads(text, parse_float=serde_f64)
    if float_parser == "exact":
        return json.loads(text)
    raise ValueError(float_parser)


def _array(a, dim):
    arr = np.asarray(a["data"], dtype=np.float64)
    if list(a["dim"]) != list(dim):
        raise ValueError(f"array dim {a['dim']} does not match size {dim}")
    return arr.reshape(dim)


def grid_from_json(g: dict) -> dict:
    """UnfinalizedSimulationGrid (src/grid/mod.rs:85-92) -> grid dict."""
    size = tuple(int(s) for s in g["size"])
    out = presets.empty(size)
    out["u"] = _array(g["u"], size)
    out["v"] = _array(g["v"], size)
    out["p"] = _array(g["pressure"], size)
    cells = g["cell_type"]
    if list(cells["dim"]) != list(size):
        raise ValueError("cell_type dim does not match size")
    for i, c in enumerate(cells["data"]):
        x, y = divmod(i, size[1])
        if c == "Fluid":
            continue
        b = c["Boundary"]
        if b == "NoSlip":
            out["kind"][x, y] = presets.NO_SLIP
        elif b == "Outflow":
            out["kind"][x, y] = presets.OUTFLOW
        elif isinstance(b, dict) and "Inflow" in b:
            out["kind"][x, y] = presets.INFLOW
            out["wall_uv"][x, y] = [float(t) for t in b["Inflow"]["velocity"]]
        elif isinstance(b, dict) and "MovingWall" in b:
            out["kind"][x, y] = presets.MOVING_WALL
            out["wall_uv"][x, y] = [float(t) for t in b["MovingWall"]["velocity"]]
        else:
            raise ValueError(f"unknown cell {c!r}")
    return out


def simulation_from_json(d: dict) -> dict:
    """UnfinalizedSimulation (src/simulation.rs:30-44) -> Simulation kwargs."""
    return {
        "grid": grid_from_json(d["grid"]),
        "cell_size": tuple(float(x) for x in d["cell_size"]),
        "delt": float(d["delt"]), "gamma": float(d["gamma"]),
        "reynolds": float(d["reynolds"]),
        "sor_absolute_epsilon": float(d["sor_absolute_epsilon"]),
        "max_iterations": int(d["max_iterations"]), "iterations": int(d["iterations"]),
        "time": float(d["time"]), "omega": float(d["omega"]),
        "initial_norm_squared": None if d.get("initial_norm_squared") is None
        else float(d["initial_norm_squared"]),
    }


def _ndarray_json(a: np.ndarray) -> dict:
    return {"v": 1, "dim": [int(a.shape[0]), int(a.shape[1])],
            "data": [float(x) for x in np.asarray(a, dtype=np.float64).ravel()]}


def _cell_json(kind: int, wall) -> object:
    if kind == presets.FLUID:
        return "Fluid"
    if kind == presets.NO_SLIP:
        return {"Boundary": "NoSlip"}
    if kind == presets.OUTFLOW:
        return {"Boundary": "Outflow"}
    if kind == presets.INFLOW:
        return {"Boundary": {"Inflow": {"velocity": [float(wall[0]), float(wall[1])]}}}
    return {"Boundary": {"MovingWall": {"velocity": [float(wall[0]), float(wall[1])]}}}


def grid_to_json(size, u, v, p, kind, wall_uv) -> dict:
    """SimulationGrid's Serialize (src/grid/mod.rs:112-125)."""
    nx, ny = size
    cells = [_cell_json(int(kind[x, y]), wall_uv[x, y]) for x in range(nx) for y in range(ny)]
    return {"size": [int(nx), int(ny)], "pressure": _ndarray_json(p), "u": _ndarray_json(u),
            "v": _ndarray_json(v),
            "cell_type": {"v": 1, "dim": [int(nx), int(ny)], "data": cells}}


def simulation_to_json(sim) -> dict:
    """Simulation's Serialize (src/simulation.rs:49-69): F, G, RHS skipped."""
    st = sim.state()
    grid = sim.grid_dict()
    return {
        "size": [int(sim.size[0]), int(sim.size[1])],
        "cell_size": [float(sim.cell_size[0]), float(sim.cell_size[1])],
        "delt": float(st["delt"]), "gamma": float(sim.gamma), "reynolds": float(sim.reynolds),
        "initial_norm_squared": float(st["initial_norm_squared"]),
        "sor_absolute_epsilon": float(sim.sor_absolute_epsilon),
        "max_iterations": int(sim.max_iterations), "iterations": int(st["iterations"]),
        "time": float(st["time"]), "omega": float(sim.omega),
        "grid": grid_to_json(sim.size, grid["u"], grid["v"], grid["p"], grid["kind"],
                             grid["wall_uv"]),
    }


def load_simulation(path_or_text, float_parser: str = "serde", **mode):
    """Simulation::from_reader (src/simulation.rs:117-120) on the GPU."""
    from .simulation import Simulation
    text = _text(path_or_text)
    return Simulation(**simulation_from_json(loads(text, float_parser)), **mode)


def load_grid(path_or_text, float_parser: str = "serde") -> dict:
    """SimulationGrid::from_reader (src/grid/mod.rs:334-341) -> grid dict."""
    return grid_from_json(loads(_text(path_or_text), float_parser))


def dumps_simulation(sim) -> str:
    return json.dumps(simulation_to_json(sim), indent=2)


def _text(path_or_text) -> str:
    if isinstance(path_or_text, Path) or (isinstance(path_or_text, str) and
                                          not path_or_text.lstrip().startswith("{")):
        return Path(path_or_text).read_text()
    return path_or_text


def save_checkpoint(sim, path) -> None:
    """Every field (F, G, RHS included), the cells and the scalar state."""
    st = sim.state()
    g = sim.grid_dict()
    np.savez(path, u=g["u"], v=g["v"], p=g["p"], f=sim.download("f"), g=sim.download("g"),
             rhs=sim.download("rhs"), kind=g["kind"], wall_uv=g["wall_uv"],
             scalars=np.array([sim.cell_size[0], sim.cell_size[1], st["delt"], sim.gamma,
                               sim.reynolds, sim.sor_absolute_epsilon, sim.max_iterations,
                               st["iterations"], st["time"], sim.omega,
                               st["initial_norm_squared"], sim.tau], dtype=np.float64))


def load_checkpoint(path, **mode):
    """Exact resume: the simulation continues bit for bit as if never saved."""
    from .simulation import Simulation
    z = np.load(path)
    s = z["scalars"]
    grid = {"kind": z["kind"], "wall_uv": z["wall_uv"], "u": z["u"], "v": z["v"], "p": z["p"]}
    sim = Simulation(grid=grid, cell_size=(s[0], s[1]), delt=s[2], gamma=s[3], reynolds=s[4],
                     sor_absolute_epsilon=s[5], max_iterations=int(s[6]), iterations=int(s[7]),
                     time=s[8], omega=s[9], initial_norm_squared=s[10], tau=s[11], **mode)
    # creation recomputes F, G, RHS from u, v (as the reference's try_from
    # does); the saved ones are what the last tick left, restore them
    sim.upload("f", z["f"])
    sim.upload("g", z["g"])
    sim.upload("rhs", z["rhs"])
    return sim
