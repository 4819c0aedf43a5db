"""Reader of NaSt2D binary ``.out`` files (the format the reference converts
into its test fixtures, python/generate_test_data.py:97-154).

Layout: two C ints (imax, jmax), then four double arrays U, V, P, T of
(imax+2) x (jmax+2) values each, x-major (``U[x][y]``), then the same number
of C int flags.  A flag with the fluid bit (16) set is a fluid cell; every
other cell is a boundary.  NaSt2D does not store which kind of boundary a cell
is; as the reference's converter does (generate_test_data.py:49-66), the left
wall's cells (x = 0, 1 <= y <= jmax) become inflow cells carrying their own
(U, V), the right wall's become outflow cells and all others no-slip.
"""
from __future__ import annotations

import struct

import numpy as np

from . import presets

FLUID_BIT = 16


def read_out(data: bytes, int_bytes: int = 4, int_type: str = "i") -> dict:
    """Parses the bytes of a .out file; returns imax, jmax and the raw arrays."""
    imax, jmax = struct.unpack_from("2" + int_type, data, 0)
    off = 2 * int_bytes
    n = (imax + 2) * (jmax + 2)
    arrays = {}
    for name in ("U", "V", "P", "T"):
        arrays[name] = np.frombuffer(data, dtype="<f8", count=n, offset=off).reshape(
            imax + 2, jmax + 2).copy()
        off += 8 * n
    flags = np.frombuffer(data, dtype="<i4" if int_bytes == 4 else "<i8", count=n,
                          offset=off).reshape(imax + 2, jmax + 2).copy()
    return {"imax": imax, "jmax": jmax, "flags": flags, **arrays}


def to_grid(out: dict) -> dict:
    """The reconstruction of the reference's converter, as a grid dict."""
    imax, jmax = out["imax"], out["jmax"]
    g = presets.empty((imax + 2, jmax + 2))
    g["u"] = out["U"].copy()
    g["v"] = out["V"].copy()
    g["p"] = out["P"].copy()
    fluid = (out["flags"] & FLUID_BIT) != 0
    kind = np.where(fluid, presets.FLUID, presets.NO_SLIP).astype(np.uint8)
    for y in range(1, jmax + 1):
        if not fluid[0, y]:
            kind[0, y] = presets.INFLOW
            g["wall_uv"][0, y] = [out["U"][0, y], out["V"][0, y]]
        if not fluid[imax + 1, y]:
            kind[imax + 1, y] = presets.OUTFLOW
    g["kind"] = kind
    return g


def load(path) -> dict:
    with open(path, "rb") as f:
        return to_grid(read_out(f.read()))
