"""The allocation-free residual norm (strm_norm_squared_noalloc).

Callers that must not allocate device memory once they run — host frameworks
whose caching allocator owns the device budget, fixed-footprint loops that
reserve all memory at start-up because cudaMalloc may synchronise the device —
get the residual norm from a fixed reduction scratch inside the library.
This test calls it through the C ABI on a live simulation's own fields and
checks it against the ordinary entry point (strm_calculate_norm_squared,
default norm over every interior cell) within the 1e-12 relative tolerance
the norm parity tests use, on two calls in a row and again after further
steps; it also checks that a grid beyond the scratch limit and a
non-positive or non-finite fluid-cell count are rejected before any GPU
work.  This file is collected last so that a failure here never hides
another test.
"""
import ctypes

import numpy as np
import pytest

from stroemung_gb300 import _lib, presets

pytestmark = pytest.mark.gpu


def _noalloc(L, view, sim, out_ptr):
    dx, dy = sim.cell_size
    return L.strm_norm_squared_noalloc(
        ctypes.cast(view["p"], ctypes.POINTER(ctypes.c_double)),
        ctypes.cast(view["rhs"], ctypes.POINTER(ctypes.c_double)),
        view["nx"], view["ny"], view["pitch"], dx, dy, sim.state()["fluid_cells"],
        ctypes.cast(out_ptr, ctypes.POINTER(ctypes.c_double)), view["stream"])


def test_noalloc_norm_matches_the_allocating_entry_point():
    import torch
    from stroemung_gb300.simulation import Simulation

    L = _lib.load()
    rects = presets.random_rectangles(300, 120, 8, 3, x_margin=20)
    g = presets.channel(300, 120, rects)
    sim = Simulation(grid=g, cell_size=(0.05, 0.05), delt=0.005, gamma=0.9, reynolds=200.0,
                     max_iterations=40, tau=0.5)
    view = sim.device_view()
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    for round_ in range(2):
        sim.run_simulation_tick()
        want = sim.calculate_norm_squared()
        got = []
        for k in range(2):  # two calls in a row, each on its own output slot
            assert _noalloc(L, view, sim, out.data_ptr() + 8 * k) == _lib.STRM_OK
            sim.synchronize()
            got.append(float(out[k].item()))
        for x in got:
            assert want > 0
            assert abs(x - want) <= 1e-12 * abs(want), (round_, x, want)
        assert got[0] == got[1]
    sim.close()


def test_noalloc_norm_rejects_grids_beyond_its_scratch():
    L = _lib.load()
    dummy = ctypes.cast(ctypes.c_void_p(256), ctypes.POINTER(ctypes.c_double))
    # 20000 x 20000 interior cells need far more than 16384 tiles
    rc = L.strm_norm_squared_noalloc(dummy, dummy, 20002, 20002, 20016, 0.1, 0.1, 1.0,
                                     dummy, None)
    assert rc == _lib.STRM_ERR_INVALID


@pytest.mark.parametrize("fluid_cells", [0.0, -5.0, float("nan"), float("inf")])
def test_noalloc_norm_rejects_bad_fluid_cell_counts(fluid_cells):
    L = _lib.load()
    dummy = ctypes.cast(ctypes.c_void_p(256), ctypes.POINTER(ctypes.c_double))
    rc = L.strm_norm_squared_noalloc(dummy, dummy, 66, 66, 80, 0.1, 0.1, fluid_cells,
                                     dummy, None)
    assert rc == _lib.STRM_ERR_INVALID
