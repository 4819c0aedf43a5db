"""Host-side mirror of the reference's Simulation / SimulationGrid API.

``Simulation`` keeps every field on the GPU and drives the sm_103a kernels
through the C ABI (include/stroemung_gpu.h).  Method names follow the Rust
crate (src/simulation.rs, src/grid/mod.rs) so that code and tests written
against the reference read the same:

    reference                                  here
    Simulation::try_from(UnfinalizedSimulation) Simulation(...) / Simulation.try_from(dict)
    sim.run_simulation_tick()                  sim.run_simulation_tick()
    sim.grid.u / .v / .pressure, sim.f/g/rhs   sim.u, sim.v, sim.pressure, sim.f, sim.g, sim.rhs
    grid.rebuild_boundary_list() after edits   sim.edit_cells(...)
    grid.pressure_range / speed_range          sim.pressure_range, sim.speed_range

Field reads download a copy ([nx, ny] float64, y contiguous); assignments
upload.  Errors map to ``BoundaryTooThinError`` and friends (src/grid/mod.rs:51-59).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _lib
from ._lib import (ARITH_EXACT, ARITH_FAST, EXEC_EAGER, EXEC_GRAPH, NORM_ALL_INTERIOR,
                   NORM_FLUID, NORM_FLUID_MEAN_FREE, PREC_FP64, PREC_MIXED, SOR_LEXICOGRAPHIC,
                   SOR_RED_BLACK, BoundaryTooThinError, NonFiniteError, StroemungError)

__all__ = ["Simulation", "BoundaryTooThinError", "NonFiniteError", "StroemungError",
           "SOR_RED_BLACK", "SOR_LEXICOGRAPHIC", "ARITH_EXACT", "ARITH_FAST", "PREC_FP64",
           "PREC_MIXED", "NORM_ALL_INTERIOR", "NORM_FLUID", "NORM_FLUID_MEAN_FREE",
           "EXEC_GRAPH", "EXEC_EAGER"]

_FIELDS = {"u": _lib.FIELD_U, "v": _lib.FIELD_V, "p": _lib.FIELD_P, "pressure": _lib.FIELD_P,
           "f": _lib.FIELD_F, "g": _lib.FIELD_G, "rhs": _lib.FIELD_RHS}


def _f64(a, shape):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != shape:
        a = a.reshape(shape)
    return a


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Simulation:
    def __init__(self, *, grid: dict, cell_size, delt: float, gamma: float, reynolds: float,
                 sor_absolute_epsilon: float = 1e-3, max_iterations: int = 100,
                 omega: float = 1.7, iterations: int = 0, time: float = 0.0,
                 initial_norm_squared=None, tau: float = 0.0, sor_order: int = SOR_RED_BLACK,
                 arithmetic: int = ARITH_EXACT, precision: int = PREC_FP64,
                 strict_eps: bool = False, inner_sweeps: int = 0, execution: int = 0,
                 norm_cells: int = NORM_ALL_INTERIOR, sweep_schedule: int = 0):
        L = _lib.load()
        kind = np.ascontiguousarray(grid["kind"], dtype=np.uint8)
        self.size = tuple(int(s) for s in kind.shape)
        nx, ny = self.size
        u = _f64(grid["u"], self.size)
        v = _f64(grid["v"], self.size)
        p = _f64(grid.get("p", grid.get("pressure")), self.size)
        wall = grid.get("wall_uv")
        wall = None if wall is None else _f64(wall, (nx, ny, 2))
        prm = _lib.Params(
            dx=float(cell_size[0]), dy=float(cell_size[1]), delt=float(delt),
            gamma=float(gamma), reynolds=float(reynolds), eps=float(sor_absolute_epsilon),
            omega=float(omega), max_iterations=int(max_iterations), iterations=int(iterations),
            time=float(time),
            initial_norm_squared=math.nan if initial_norm_squared is None
            else float(initial_norm_squared),
            tau=float(tau))
        self.cell_size = (prm.dx, prm.dy)
        self.gamma, self.reynolds, self.omega = prm.gamma, prm.reynolds, prm.omega
        self.sor_absolute_epsilon = prm.eps
        self.max_iterations = prm.max_iterations
        self.tau = prm.tau
        h = ctypes.c_void_p()
        bad = ctypes.c_int64(-1)
        rc = L.strm_create(ctypes.byref(prm), nx, ny,
                           kind.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                           _dp(wall) if wall is not None else None, _dp(u), _dp(v), _dp(p),
                           ctypes.byref(h), ctypes.byref(bad))
        if rc == _lib.STRM_ERR_THIN_WALL:
            raise BoundaryTooThinError(rc, f"{_lib.last_error()} at {divmod(bad.value, ny)}")
        _lib.check(rc)
        self._h = h
        # host copies of what the device keeps only in compiled form
        self._kind = kind.copy()
        self._wall = np.zeros((nx, ny, 2)) if wall is None else wall.copy()
        self.set_mode(sor_order=sor_order, arithmetic=arithmetic, precision=precision,
                      strict_eps=strict_eps, inner_sweeps=inner_sweeps, execution=execution,
                      norm_cells=norm_cells, sweep_schedule=sweep_schedule)

    @classmethod
    def from_json(cls, path_or_text, float_parser: str = "serde", **mode):
        """Simulation::from_reader (src/simulation.rs:117-120)."""
        from . import jsonio
        return jsonio.load_simulation(path_or_text, float_parser, **mode)

    def to_json(self) -> str:
        """Simulation's serde layout (src/simulation.rs:49-69)."""
        from . import jsonio
        return jsonio.dumps_simulation(self)

    def grid_dict(self) -> dict:
        """Host copy of the grid: kind, wall_uv, u, v, p."""
        return {"kind": self._kind.copy(), "wall_uv": self._wall.copy(), "u": self.download("u"),
                "v": self.download("v"), "p": self.download("p")}

    @classmethod
    def try_from(cls, unfinalized: dict, **mode):
        """From the reference's UnfinalizedSimulation layout (src/simulation.rs:30-44)."""
        return cls(grid=unfinalized["grid"], cell_size=unfinalized["cell_size"],
                   delt=unfinalized["delt"], gamma=unfinalized["gamma"],
                   reynolds=unfinalized["reynolds"],
                   sor_absolute_epsilon=unfinalized["sor_absolute_epsilon"],
                   max_iterations=unfinalized["max_iterations"], omega=unfinalized["omega"],
                   iterations=unfinalized.get("iterations", 0),
                   time=unfinalized.get("time", 0.0),
                   initial_norm_squared=unfinalized.get("initial_norm_squared"), **mode)

    # ---- lifetime ---------------------------------------------------------
    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().strm_destroy(h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- configuration ---------------------------------------------------
    def set_mode(self, *, sor_order=SOR_RED_BLACK, arithmetic=ARITH_EXACT, precision=PREC_FP64,
                 strict_eps=False, inner_sweeps=0, execution=0, norm_cells=NORM_ALL_INTERIOR,
                 sweep_schedule=0):
        rule = int(strict_eps) if not isinstance(strict_eps, bool) else int(strict_eps)
        m = _lib.Mode(sor_order=sor_order, arithmetic=arithmetic, precision=precision,
                      strict_eps=rule, inner_sweeps=inner_sweeps,
                      execution=execution, norm_cells=norm_cells, sweep_schedule=sweep_schedule)
        _lib.check(_lib.load().strm_set_mode(self._h, ctypes.byref(m)))
        self.mode = {"sor_order": sor_order, "arithmetic": arithmetic, "precision": precision,
                     "strict_eps": rule, "inner_sweeps": inner_sweeps,
                     "execution": execution, "norm_cells": norm_cells,
                     "sweep_schedule": sweep_schedule}

    def residual_history(self) -> np.ndarray:
        """(sweeps, norm_squared) rows of the last pressure solve."""
        n = ctypes.c_int(0)
        L = _lib.load()
        _lib.check(L.strm_residual_history(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros((max(n.value, 1), 2))
        _lib.check(L.strm_residual_history(self._h, _dp(out), n.value, ctypes.byref(n)))
        return out[:n.value]

    def autotune_sweeps(self, reps: int = 5):
        """Times every FP32 sweep schedule on this grid, keeps the fastest;
        returns (schedule, {schedule: ms per sweep})."""
        best = ctypes.c_int(0)
        ms = (ctypes.c_double * _lib.SWEEPS_COUNT)()
        _lib.check(_lib.load().strm_autotune_sweeps(self._h, int(reps), ctypes.byref(best), ms))
        self.mode["sweep_schedule"] = best.value
        return best.value, {v: ms[v] for v in range(1, _lib.SWEEPS_COUNT)}

    # ---- the timestep (src/simulation.rs:324-333) --------------------------
    def run_simulation_tick(self):
        it = ctypes.c_uint32(0)
        ns = ctypes.c_double(0.0)
        _lib.check(_lib.load().strm_tick(self._h, ctypes.byref(it), ctypes.byref(ns)))
        return it.value, ns.value

    def tick_prepare(self):
        """First half of a tick: time step, boundary pass, F/G and RHS."""
        _lib.check(_lib.load().strm_tick_prepare(self._h))

    def tick_solve(self):
        """Second half: pressure solve, velocity update, time bookkeeping;
        returns what run_simulation_tick returns."""
        it = ctypes.c_uint32(0)
        ns = ctypes.c_double(0.0)
        _lib.check(_lib.load().strm_tick_solve(self._h, ctypes.byref(it), ctypes.byref(ns)))
        return it.value, ns.value

    def step_n(self, n: int):
        """n ticks with one host synchronisation; returns per-tick
        (sor_iterations, norm_squared, delt, converged)."""
        stats = (_lib.StepStats * max(n, 1))()
        _lib.check(_lib.load().strm_step_n(self._h, int(n), stats))
        return [(s.sor_iterations, s.norm_squared, s.delt, bool(s.converged))
                for s in stats[:n]]

    # ---- fields -----------------------------------------------------------
    def download(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.size, dtype=np.float64)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == \
            self.size[0] * self.size[1]
        _lib.check(_lib.load().strm_download(self._h, _FIELDS[name], _dp(out)))
        return out

    def upload(self, name: str, a) -> None:
        a = _f64(a, self.size)
        _lib.check(_lib.load().strm_upload(self._h, _FIELDS[name], _dp(a)))

    u = property(lambda s: s.download("u"), lambda s, a: s.upload("u", a))
    v = property(lambda s: s.download("v"), lambda s, a: s.upload("v", a))
    pressure = property(lambda s: s.download("p"), lambda s, a: s.upload("p", a))
    f = property(lambda s: s.download("f"), lambda s, a: s.upload("f", a))
    g = property(lambda s: s.download("g"), lambda s, a: s.upload("g", a))
    rhs = property(lambda s: s.download("rhs"), lambda s, a: s.upload("rhs", a))

    def cells(self):
        """(kinds, edge codes) of every cell, [nx, ny] uint8."""
        k = np.empty(self.size, np.uint8)
        e = np.empty(self.size, np.uint8)
        _lib.check(_lib.load().strm_download_cells(
            self._h, k.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
            e.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return k, e

    @property
    def cell_type(self):
        return self.cells()[0]

    def edit_cells(self, xs, ys, kinds, wall_uv=None):
        """The GUI paint + rebuild_boundary_list path with rollback
        (src/lib.rs:38-78).  Raises BoundaryTooThinError, state unchanged."""
        xs = np.ascontiguousarray(xs, dtype=np.int32)
        ys = np.ascontiguousarray(ys, dtype=np.int32)
        kinds = np.ascontiguousarray(np.broadcast_to(np.asarray(kinds, np.uint8), xs.shape))
        w = None
        if wall_uv is not None:
            w = np.ascontiguousarray(np.broadcast_to(np.asarray(wall_uv, np.float64),
                                                     xs.shape + (2,)))
        bad = ctypes.c_int64(-1)
        _lib.check(_lib.load().strm_edit_cells(
            self._h, len(xs), xs.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            ys.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            kinds.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
            _dp(w) if w is not None else None, ctypes.byref(bad)))
        self._kind[xs, ys] = kinds
        self._wall[xs, ys] = 0.0 if w is None else w

    # ---- scalar state -------------------------------------------------------
    def state(self) -> dict:
        s = _lib.State()
        _lib.check(_lib.load().strm_get_state(self._h, ctypes.byref(s)))
        return {"time": s.time, "iterations": s.iterations, "delt": s.delt,
                "initial_norm_squared": s.initial_norm_squared, "fluid_cells": s.fluid_cells,
                "pressure_range": (s.pressure_range[0], s.pressure_range[1]),
                "speed_range": (s.speed_range[0], s.speed_range[1]),
                "last_sor_iterations": s.last_sor_iterations,
                "last_norm_squared": s.last_norm_squared,
                "last_converged": bool(s.last_converged)}

    time = property(lambda s: s.state()["time"])
    iterations = property(lambda s: s.state()["iterations"])
    initial_norm_squared = property(lambda s: s.state()["initial_norm_squared"])
    pressure_range = property(lambda s: s.state()["pressure_range"])
    speed_range = property(lambda s: s.state()["speed_range"])
    delt = property(lambda s: s.state()["delt"])

    # ---- individual phases -------------------------------------------------
    def set_boundary_u_and_v(self):
        _lib.check(_lib.load().strm_set_boundary_u_and_v(self._h))

    def calculate_f_g_rhs(self):
        _lib.check(_lib.load().strm_calculate_f_g_rhs(self._h))

    def copy_pressure_to_boundaries(self):
        _lib.check(_lib.load().strm_copy_pressure_to_boundaries(self._h))

    def calculate_norm_squared(self) -> float:
        ns = ctypes.c_double(0.0)
        _lib.check(_lib.load().strm_calculate_norm_squared(self._h, ctypes.byref(ns)))
        return ns.value

    def set_u_and_v(self):
        _lib.check(_lib.load().strm_set_u_and_v(self._h))

    def sor_sweeps(self, n: int, wait: bool = True):
        """n pressure iterations with no stop test; returns the last norm
        (None when wait is False: the work is only queued)."""
        if not wait:
            _lib.check(_lib.load().strm_sor_sweeps(self._h, int(n), None))
            return None
        ns = ctypes.c_double(0.0)
        _lib.check(_lib.load().strm_sor_sweeps(self._h, int(n), ctypes.byref(ns)))
        return ns.value

    def synchronize(self):
        _lib.check(_lib.load().strm_synchronize(self._h))

    def calculate_pressure_range(self):
        _lib.check(_lib.load().strm_calculate_pressure_range(self._h))

    def calculate_speed_range(self):
        _lib.check(_lib.load().strm_calculate_speed_range(self._h))

    def render(self, color_type: str = "pressure") -> np.ndarray:
        """render_simulation (src/visualization.rs:79-105) on the GPU:
        [ny, nx, 4] uint8 RGBA, image row = y."""
        ct = {"pressure": 0, "speed": 1}[color_type]
        out = np.empty((self.size[1], self.size[0], 4), dtype=np.uint8)
        _lib.check(_lib.load().strm_render_rgba(
            self._h, ct, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return out

    def device_view(self) -> dict:
        dv = _lib.DeviceView()
        _lib.check(_lib.load().strm_device_view_get(self._h, ctypes.byref(dv)))
        return {k: getattr(dv, k) for k, _ in dv._fields_}


def host_classify(kind: np.ndarray):
    """Edge codes of every cell on the host; raises BoundaryTooThinError."""
    kind = np.ascontiguousarray(kind, dtype=np.uint8)
    nx, ny = kind.shape
    edges = np.zeros_like(kind)
    fc = ctypes.c_double(0)
    bad = ctypes.c_int64(-1)
    rc = _lib.load().strm_host_classify(nx, ny, kind.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                        edges.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                        ctypes.byref(fc), ctypes.byref(bad))
    if rc == _lib.STRM_ERR_THIN_WALL:
        raise BoundaryTooThinError(rc, f"thin wall at {divmod(bad.value, ny)}")
    _lib.check(rc)
    return edges, fc.value


def host_boundary_pass(kind, wall_uv, u, v):
    """The compiled boundary program applied on the host: returns
    (u', v', restore_u, restore_v)."""
    kind = np.ascontiguousarray(kind, dtype=np.uint8)
    nx, ny = kind.shape
    u = np.array(u, dtype=np.float64, order="C")
    v = np.array(v, dtype=np.float64, order="C")
    ru = np.full((nx, ny), np.nan)
    rv = np.full((nx, ny), np.nan)
    w = None if wall_uv is None else _f64(wall_uv, (nx, ny, 2))
    _lib.check(_lib.load().strm_host_boundary_pass(
        nx, ny, kind.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
        _dp(w) if w is not None else None, _dp(u), _dp(v), _dp(ru), _dp(rv)))
    return u, v, ru, rv


def write_png(path, rgba: np.ndarray) -> None:
    """Writes an [h, w, 4] uint8 image as a PNG (zlib, no imaging library)."""
    import struct
    import zlib
    h, w, _ = rgba.shape
    raw = b"".join(b"\x00" + np.ascontiguousarray(rgba[y]).tobytes() for y in range(h))

    def chunk(tag, data):
        return (struct.pack(">I", len(data)) + tag + data +
                struct.pack(">I", zlib.crc32(tag + data) & 0xffffffff))
    png = (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
           chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(png)
