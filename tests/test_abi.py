"""The C-ABI library builds, loads and exports every entry point the public
header declares; without a GPU it refuses to create a simulation (no host
fallback)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from stroemung_gb300 import _lib, presets

HEADERS = sorted((Path(__file__).resolve().parent.parent / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\bint\s+(strm_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_the_expected_surface():
    names = declared_functions()
    for must in ("strm_create", "strm_tick", "strm_step_n", "strm_download", "strm_upload",
                 "strm_edit_cells", "strm_destroy", "strm_last_error"):
        assert must in names


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    for name in declared_functions():
        assert hasattr(L, name), name
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature"
    assert set(_lib.SIGNATURES) == set(declared_functions())
    assert L.strm_abi_version() == 1


def test_struct_sizes_match_header_layout():
    # strm_params: 7 doubles, 2 uint32, 3 doubles
    assert ctypes.sizeof(_lib.Params) == 7 * 8 + 2 * 4 + 3 * 8
    assert ctypes.sizeof(_lib.Mode) == 8 * 4
    assert ctypes.sizeof(_lib.StepStats) == 24


def test_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from stroemung_gb300.simulation import Simulation, StroemungError
    g = presets.simple_inflow((4, 3))
    with pytest.raises(StroemungError) as ei:
        Simulation(grid=g, cell_size=(0.1, 0.2), delt=0.005, gamma=0.9, reynolds=100.0)
    assert ei.value.code in (_lib.STRM_ERR_NO_DEVICE, _lib.STRM_ERR_CUDA)


def test_conv_launch_shape_rejects_values_out_of_range():
    """strm_nn_tune_conv_tma only records the launch shape (no device call):
    CTAs per SM 0..8, stages 0 or 2..32, tiles per CTA 0..64, rows 0 or 1."""
    L = _lib.load()
    for bad in ((-1, 0, 1, 1), (9, 0, 1, 1), (0, 1, 1, 1), (0, 33, 1, 1), (0, -2, 1, 1),
                (0, 0, 65, 1), (0, 0, -1, 1), (0, 0, 1, 2), (0, 0, 1, -1)):
        assert L.strm_nn_tune_conv_tma(*bad) == 6, bad
    for good in ((0, 0, 0, 0), (2, 6, 1, 1), (1, 32, 0, 1), (8, 2, 64, 0)):
        assert L.strm_nn_tune_conv_tma(*good) == 0, good
    assert L.strm_nn_tune_conv_tma(0, 0, 0, 1) == 0


def test_programmatic_launch_switch_returns_the_previous_setting():
    """strm_set_programmatic_launch only records a process-wide setting for
    graphs built afterwards (no device call): on by default, any nonzero
    value means on, and each call returns the setting it replaced."""
    L = _lib.load()
    prev = L.strm_set_programmatic_launch(0)
    try:
        assert prev in (0, 1)
        assert L.strm_set_programmatic_launch(7) == 0
        assert L.strm_set_programmatic_launch(1) == 1
    finally:
        L.strm_set_programmatic_launch(prev)
