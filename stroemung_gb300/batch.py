"""Batches of independent simulations stepped by one CUDA graph
(strm_batch_* in include/stroemung_gpu.h): the members' pressure solves run
as one WHILE loop of table-driven kernels or as one persistent cooperative
kernel, each member ending exactly where stepping it alone ends.  No reference counterpart (the crate steps one
simulation)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


class Batch:
    def __init__(self, sims, inner_sweeps: int = 0):
        L = _lib.load()
        self.sims = list(sims)
        arr = (ctypes.c_void_p * len(self.sims))(*[s._h.value for s in self.sims])
        h = ctypes.c_void_p()
        _lib.check(L.strm_batch_create(arr, len(self.sims), int(inner_sweeps), ctypes.byref(h)))
        self._h = h

    def step(self, n: int = 1) -> np.ndarray:
        """n steps of every member; returns a structured array [member][step]
        with sor_iterations, norm_squared, delt, converged."""
        m = len(self.sims)
        buf = (_lib.StepStats * (m * max(n, 1)))()
        _lib.check(_lib.load().strm_batch_step(self._h, int(n), ctypes.cast(buf, ctypes.c_void_p)))
        dt = np.dtype([("sor_iterations", np.uint32), ("norm_squared", np.float64),
                       ("delt", np.float64), ("converged", np.uint32)])
        out = np.zeros((m, n), dt)
        for k in range(m):
            for i in range(n):
                s = buf[k * n + i]
                out[k, i] = (s.sor_iterations, s.norm_squared, s.delt, s.converged)
        return out

    def prepare(self) -> None:
        """First half of a batch step: every member's boundary pass, time
        step, F/G and RHS (the members' pressures may be changed before
        solve)."""
        _lib.check(_lib.load().strm_batch_prepare(self._h))

    def solve(self) -> np.ndarray:
        """Second half: the pressure solves and velocity updates; returns
        one record per member (as step(1)[:, 0])."""
        m = len(self.sims)
        buf = (_lib.StepStats * m)()
        _lib.check(_lib.load().strm_batch_solve(self._h, ctypes.cast(buf, ctypes.c_void_p)))
        dt = np.dtype([("sor_iterations", np.uint32), ("norm_squared", np.float64),
                       ("delt", np.float64), ("converged", np.uint32)])
        out = np.zeros(m, dt)
        for k in range(m):
            s = buf[k]
            out[k] = (s.sor_iterations, s.norm_squared, s.delt, s.converged)
        return out

    def set_schedule(self, schedule: int) -> None:
        _lib.check(_lib.load().strm_batch_set_schedule(self._h, int(schedule)))

    def set_solver(self, persistent: bool, wait_limit: int = 0) -> None:
        """persistent: the members' pressure solves run as one persistent
        cooperative kernel per step (grid barriers between its phases, each
        wait bounded by wait_limit polls, 0 = about a second or two) instead
        of the graph's WHILE loop; results are identical."""
        solver = _lib.BATCH_PERSISTENT if persistent else _lib.BATCH_GRAPH_LOOP
        _lib.check(_lib.load().strm_batch_set_solver(self._h, solver, int(wait_limit)))

    def autotune(self, reps: int = 2):
        """Times whole batch steps under every blocked schedule (members'
        state restored), keeps the fastest; returns (schedule, {schedule: ms})."""
        best = ctypes.c_int(0)
        ms = (ctypes.c_double * _lib.SWEEPS_COUNT)()
        _lib.check(_lib.load().strm_batch_autotune(self._h, int(reps), ctypes.byref(best), ms))
        return best.value, {v: ms[v] for v in range(2, _lib.SWEEPS_COUNT)}

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().strm_batch_destroy(h)
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
