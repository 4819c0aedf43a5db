"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

The oracle (``stroemung_oracle.c``) restates the reference solver's FP64
timestep (wickedchicken/stroemung ``src/math.rs``, ``src/simulation.rs``,
``src/grid/mod.rs``) with its operation and loop order.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
this module; the product package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libstroemung_oracle.so"

FLUID, NO_SLIP, OUTFLOW, INFLOW, MOVING_WALL = 0, 1, 2, 3, 4
LEXICOGRAPHIC, RED_BLACK = 0, 1
FIELDS = {"u": 0, "v": 1, "p": 2, "f": 3, "g": 4, "rhs": 5}

_dp = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int),
        ("ny", ctypes.c_int),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("delt", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("reynolds", ctypes.c_double),
        ("eps", ctypes.c_double),
        ("omega", ctypes.c_double),
        ("max_iterations", ctypes.c_uint32),
        ("iterations", ctypes.c_uint32),
        ("time", ctypes.c_double),
        ("initial_norm_squared", ctypes.c_double),
        ("has_initial_norm", ctypes.c_int),
        ("tau", ctypes.c_double),
        ("sor_order", ctypes.c_int),
        ("strict_eps", ctypes.c_int),
    ]


def build() -> Path:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        for name in ("orc_du2dx", "orc_dv2dy"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [_dp, ctypes.c_double, ctypes.c_double]
        for name in ("orc_duvdx", "orc_duvdy"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_double]
        L.orc_laplacian.restype = ctypes.c_double
        L.orc_laplacian.argtypes = [_dp, ctypes.c_double, ctypes.c_double]
        L.orc_residual.restype = ctypes.c_double
        L.orc_residual.argtypes = [_dp, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        for name in ("orc_calculate_f", "orc_calculate_g"):
            getattr(L, name).restype = ctypes.c_double
            getattr(L, name).argtypes = [_dp, _dp] + [ctypes.c_double] * 5
        L.orc_classify.restype = ctypes.c_int
        L.orc_classify.argtypes = [ctypes.c_int, ctypes.c_int, _u8p, _u8p, _dp,
                                   ctypes.POINTER(ctypes.c_int64)]
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(OrcParams), _u8p, _dp, _dp, _dp, _dp,
                                 ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int64)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_tick.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32), _dp]
        L.orc_get_field.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_set_field.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_get_edges.argtypes = [ctypes.c_void_p, _u8p]
        L.orc_get_state.argtypes = [ctypes.c_void_p, _dp]
        for name in ("orc_set_boundary_u_and_v", "orc_calculate_f_and_g", "orc_calculate_rhs",
                     "orc_copy_pressure_to_boundaries", "orc_set_u_and_v", "orc_adapt_dt",
                     "orc_calculate_pressure_range", "orc_calculate_speed_range"):
            getattr(L, name).argtypes = [ctypes.c_void_p]
        L.orc_calculate_norm_squared.restype = ctypes.c_double
        L.orc_calculate_norm_squared.argtypes = [ctypes.c_void_p]
        L.orc_solve_sor.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32), _dp]
        L.orc_tick_timed.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _dp]
        L.orc_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_render.argtypes = [ctypes.c_void_p, ctypes.c_int, _u8p]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _window(a) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    assert a.shape == (3, 3)
    return a


def du2dx(u, delx, gamma):
    u = _window(u)
    return lib().orc_du2dx(_d(u), delx, gamma)


def duvdx(u, v, delx, gamma):
    u, v = _window(u), _window(v)
    return lib().orc_duvdx(_d(u), _d(v), delx, gamma)


def duvdy(u, v, dely, gamma):
    u, v = _window(u), _window(v)
    return lib().orc_duvdy(_d(u), _d(v), dely, gamma)


def dv2dy(v, dely, gamma):
    v = _window(v)
    return lib().orc_dv2dy(_d(v), dely, gamma)


def laplacian(e, delx, dely):
    e = _window(e)
    return lib().orc_laplacian(_d(e), delx, dely)


def calculate_f(u, v, delx, dely, delt, gamma, reynolds):
    u, v = _window(u), _window(v)
    return lib().orc_calculate_f(_d(u), _d(v), delx, dely, delt, gamma, reynolds)


def calculate_g(u, v, delx, dely, delt, gamma, reynolds):
    u, v = _window(u), _window(v)
    return lib().orc_calculate_g(_d(u), _d(v), delx, dely, delt, gamma, reynolds)


def classify(kind: np.ndarray):
    """Returns (edge codes, fluid_cells, bad_index or None)."""
    kind = np.ascontiguousarray(kind, dtype=np.uint8)
    nx, ny = kind.shape
    edge = np.zeros_like(kind)
    fc = ctypes.c_double(0.0)
    bad = ctypes.c_int64(-1)
    rc = lib().orc_classify(nx, ny, kind.ctypes.data_as(_u8p), edge.ctypes.data_as(_u8p),
                            ctypes.byref(fc), ctypes.byref(bad))
    return edge, fc.value, (bad.value if rc else None)


class OracleError(RuntimeError):
    pass


class OracleSim:
    """One simulation held by the C oracle; fields are [nx, ny] float64."""

    def __init__(self, *, kind, u, v, p, dx, dy, delt, gamma, reynolds, eps=1e-3,
                 omega=1.7, max_iterations=100, iterations=0, time=0.0,
                 initial_norm_squared=None, tau=0.0, sor_order=LEXICOGRAPHIC,
                 strict_eps=False, wall_uv=None):
        kind = np.ascontiguousarray(kind, dtype=np.uint8)
        nx, ny = kind.shape
        self.nx, self.ny = nx, ny
        prm = OrcParams(nx=nx, ny=ny, dx=dx, dy=dy, delt=delt, gamma=gamma, reynolds=reynolds,
                        eps=eps, omega=omega, max_iterations=max_iterations,
                        iterations=iterations, time=time,
                        initial_norm_squared=0.0 if initial_norm_squared is None
                        else initial_norm_squared,
                        has_initial_norm=0 if initial_norm_squared is None else 1,
                        tau=tau, sor_order=sor_order, strict_eps=1 if strict_eps else 0)
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(nx, ny) for a in (u, v, p)]
        wall = None
        if wall_uv is not None:
            wall = np.ascontiguousarray(wall_uv, dtype=np.float64).reshape(nx, ny, 2)
        status = ctypes.c_int(0)
        bad = ctypes.c_int64(-1)
        h = lib().orc_create(ctypes.byref(prm), kind.ctypes.data_as(_u8p),
                             _d(wall) if wall is not None else None,
                             _d(arrs[0]), _d(arrs[1]), _d(arrs[2]),
                             ctypes.byref(status), ctypes.byref(bad))
        if not h:
            raise OracleError(f"thin boundary at {divmod(bad.value, ny)}")
        self._h = ctypes.c_void_p(h)
        self.kind = kind

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().orc_destroy(h)
            self._h = None

    def tick(self):
        it = ctypes.c_uint32(0)
        ns = ctypes.c_double(0.0)
        lib().orc_tick(self._h, ctypes.byref(it), ctypes.byref(ns))
        return it.value, ns.value

    def field(self, name: str) -> np.ndarray:
        out = np.empty((self.nx, self.ny), dtype=np.float64)
        lib().orc_get_field(self._h, FIELDS[name], _d(out))
        return out

    def set_field(self, name: str, a) -> None:
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(self.nx, self.ny)
        lib().orc_set_field(self._h, FIELDS[name], _d(a))

    def edges(self) -> np.ndarray:
        out = np.empty((self.nx, self.ny), dtype=np.uint8)
        lib().orc_get_edges(self._h, out.ctypes.data_as(_u8p))
        return out

    def state(self) -> dict:
        out = np.empty(8, dtype=np.float64)
        lib().orc_get_state(self._h, _d(out))
        return {"time": out[0], "iterations": int(out[1]), "initial_norm_squared": out[2],
                "delt": out[3], "pressure_range": (out[4], out[5]),
                "speed_range": (out[6], out[7])}

    # phase-level access, for kernel-by-kernel parity
    def set_boundary_u_and_v(self):
        lib().orc_set_boundary_u_and_v(self._h)

    def calculate_f_and_g(self):
        lib().orc_calculate_f_and_g(self._h)

    def calculate_rhs(self):
        lib().orc_calculate_rhs(self._h)

    def copy_pressure_to_boundaries(self):
        lib().orc_copy_pressure_to_boundaries(self._h)

    def norm_squared(self) -> float:
        return lib().orc_calculate_norm_squared(self._h)

    def solve_sor(self):
        it = ctypes.c_uint32(0)
        ns = ctypes.c_double(0.0)
        lib().orc_solve_sor(self._h, ctypes.byref(it), ctypes.byref(ns))
        return it.value, ns.value

    def set_u_and_v(self):
        lib().orc_set_u_and_v(self._h)

    def render(self, color_type: int) -> np.ndarray:
        """src/visualization.rs colour map: [ny, nx, 4] uint8 (0 pressure, 1 speed)."""
        out = np.zeros((self.ny, self.nx, 4), dtype=np.uint8)
        lib().orc_render(self._h, int(color_type), out.ctypes.data_as(_u8p))
        return out

    def tick_timed(self, max_iterations_cap: int = 0):
        """(seconds before the solve, seconds in it, iterations, seconds after)."""
        out = np.zeros(4)
        lib().orc_tick_timed(self._h, int(max_iterations_cap), _d(out))
        return float(out[0]), float(out[1]), int(out[2]), float(out[3])

    def adapt_dt(self):
        lib().orc_adapt_dt(self._h)

    def set_threads(self, n: int):
        """Threads of the red-black sweeps and the norm (timing only; 1 runs
        the serial loops)."""
        lib().orc_set_threads(self._h, int(n))
