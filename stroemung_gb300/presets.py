"""Grid builders.

``empty``, ``simple_inflow`` and ``obstacle`` restate the reference's presets
(src/grid/presets.rs:8-87).  ``channel``, ``random_rectangles`` and ``cavity``
build the synthetic workloads this project measures on: a channel with
axis-aligned rectangular obstacles and a lid-driven cavity.

A grid here is a plain dict of host arrays, all [nx, ny] with the one-cell
ring included and y the contiguous axis (src/types.rs:12-19):

    kind     uint8   FLUID / NO_SLIP / OUTFLOW / INFLOW / MOVING_WALL
    wall_uv  float64 [nx, ny, 2] velocity of inflow and moving-wall cells
    u, v, p  float64
"""
from __future__ import annotations

import math

import numpy as np

FLUID, NO_SLIP, OUTFLOW, INFLOW, MOVING_WALL = 0, 1, 2, 3, 4


def _grid(nx: int, ny: int) -> dict:
    return {
        "kind": np.zeros((nx, ny), dtype=np.uint8),
        "wall_uv": np.zeros((nx, ny, 2), dtype=np.float64),
        "u": np.zeros((nx, ny), dtype=np.float64),
        "v": np.zeros((nx, ny), dtype=np.float64),
        "p": np.zeros((nx, ny), dtype=np.float64),
    }


def empty(size) -> dict:
    """All fluid, zero fields (src/grid/presets.rs:8-17)."""
    return _grid(int(size[0]), int(size[1]))


def simple_inflow(size, inflow=(1.0, 0.0)) -> dict:
    """No-slip top and bottom rows, inflow on x=0, outflow on x=nx-1
    (src/grid/presets.rs:19-40)."""
    nx, ny = int(size[0]), int(size[1])
    g = _grid(nx, ny)
    k = g["kind"]
    k[:, 0] = NO_SLIP
    k[:, ny - 1] = NO_SLIP
    k[0, 1:ny - 1] = INFLOW
    g["wall_uv"][0, 1:ny - 1] = inflow
    k[nx - 1, 1:ny - 1] = OUTFLOW
    return g


def _draw_circle(kind: np.ndarray, x: int, y: int, radius: float) -> None:
    """src/grid/presets.rs:42-62, including its half-open loop bounds."""
    xs, ys = kind.shape
    r = int(radius)
    for xi in range(max(x - r, 0), x + r):
        if xi >= xs:
            continue
        for yi in range(max(y - r, 0), y + r):
            if yi >= ys:
                continue
            if math.sqrt(float((xi - x) ** 2 + (yi - y) ** 2)) < radius:
                kind[xi, yi] = NO_SLIP


def obstacle(size) -> dict:
    """simple_inflow plus a radius-5 disc at (20, ny/2) (src/grid/presets.rs:64-87)."""
    g = simple_inflow(size)
    _draw_circle(g["kind"], 20, int(size[1]) // 2, 5.0)
    return g


def channel(imax: int, jmax: int, rects=(), u0: float = 1.0) -> dict:
    """Channel of imax x jmax interior cells: no-slip walls top and bottom,
    inflow (1, 0) on the left, outflow on the right, no-slip rectangles
    ``(x0, y0, w, h)`` in ring coordinates, u = u0 on fluid cells."""
    g = simple_inflow((imax + 2, jmax + 2))
    k = g["kind"]
    for (x0, y0, w, h) in rects:
        k[x0:x0 + w, y0:y0 + h] = NO_SLIP
    g["u"][k == FLUID] = u0
    return g


def random_rectangles(imax: int, jmax: int, count: int, seed: int, side=(4, 32),
                      gap: int = 2, x_margin: int = 64, y_margin: int = 2,
                      max_tries: int = 100000):
    """Seeded rectangles with sides uniform in [side[0], side[1]], at least
    ``gap`` fluid cells from each other, ``x_margin`` cells from the inflow and
    outflow columns and ``y_margin`` cells from the walls, so that no
    boundary cell has fluid on opposite sides."""
    rng = np.random.default_rng(seed)
    rects = []
    lo_x, hi_x = 1 + x_margin, imax + 1 - x_margin
    lo_y, hi_y = 1 + y_margin, jmax + 1 - y_margin
    tries = 0
    while len(rects) < count:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"placed only {len(rects)} of {count} rectangles")
        w = int(rng.integers(side[0], side[1] + 1))
        h = int(rng.integers(side[0], side[1] + 1))
        if hi_x - w <= lo_x or hi_y - h <= lo_y:
            continue
        x0 = int(rng.integers(lo_x, hi_x - w + 1))
        y0 = int(rng.integers(lo_y, hi_y - h + 1))
        ok = True
        for (a, b, c, d) in rects:
            if (x0 < a + c + gap and a < x0 + w + gap and
                    y0 < b + d + gap and b < y0 + h + gap):
                ok = False
                break
        if ok:
            rects.append((x0, y0, w, h))
    return rects


def cavity(n: int, lid=(1.0, 0.0)) -> dict:
    """Lid-driven cavity of n x n interior cells: the top row (y = 0; north
    is y-1) is a moving wall with velocity ``lid``, the other walls no-slip,
    fields zero."""
    g = _grid(n + 2, n + 2)
    k = g["kind"]
    k[0, :] = NO_SLIP
    k[n + 1, :] = NO_SLIP
    k[:, n + 1] = NO_SLIP
    k[:, 0] = MOVING_WALL
    g["wall_uv"][:, 0] = lid
    return g


def square_obstacle_channel() -> dict:
    """The 100 x 20 channel with one 4 x 4 no-slip block around interior
    cell (20, 10): ring coordinates x in [19, 22], y in [9, 12]."""
    return channel(100, 20, rects=[(19, 9, 4, 4)])
