"""Mixed-precision particle positions: an int32 cell index plus 16-bit offsets.

Layout (the input of ``asg_load_particles_quantised`` / ``asg_smooth_quantised``):

* a cubic grid of ``grid``^3 cells of side ``cell_size`` whose corner is at
  ``left`` (the buffered cube's lower edge) and which covers ``[left, right)``;
* ``cell``: int32 per particle, ``(cz * grid + cy) * grid + cx``;
* ``off``: uint16 per particle and axis, the position inside the cell in units
  of ``cell_size / 65536``.

Decoding is defined as float32 arithmetic, each product and sum rounded to
nearest in this order:

    x = (left + cell_size * cx) + off_x * (cell_size / 65536)

``dequantise`` below is that definition on the host; the device decode performs
the same operations, so both give the same float32 positions.  With 4-unit
cells and coordinates below 1024 in magnitude every decoded position is exact
(a multiple of 2^-14 with at most 24 significant bits).

There is no counterpart in the reference, whose particles always carry float
positions (basic_types.h:10-15).
"""
from __future__ import annotations

import numpy as np

__all__ = ["quantise", "dequantise", "grid_size"]


def grid_size(left: float, right: float, cell_size: float) -> int:
    """Cells per axis of a grid of side ``cell_size`` covering [left, right)."""
    g = int(np.ceil((float(right) - float(left)) / float(cell_size)))
    while np.float32(left) + np.float32(cell_size) * np.float32(g) < np.float32(right):
        g += 1
    return g


def quantise(x: np.ndarray, left: float, right: float, cell_size: float = 4.0):
    """Positions (n, 3) -> (cell int32 (n,), off uint16 (n, 3), grid).

    Offsets are truncated toward the cell's lower corner (resolution
    cell_size / 65536)."""
    x = np.asarray(x, np.float64)
    grid = grid_size(left, right, cell_size)
    rel = (x - float(left)) / float(cell_size)
    ci = np.clip(np.floor(rel), 0, grid - 1).astype(np.int64)
    off = np.clip(np.floor((rel - ci) * 65536.0), 0, 65535).astype(np.uint16)
    cell = ((ci[:, 2] * grid + ci[:, 1]) * grid + ci[:, 0]).astype(np.int32)
    return cell, off, grid


def dequantise(cell: np.ndarray, off: np.ndarray, grid: int, left: float,
               cell_size: float = 4.0) -> np.ndarray:
    """The decode definition in float32 (same operations and order as the device)."""
    cell = np.asarray(cell, np.int64)
    cx = (cell % grid).astype(np.float32)
    cy = ((cell // grid) % grid).astype(np.float32)
    cz = (cell // (grid * grid)).astype(np.float32)
    cs = np.float32(cell_size)
    lf = np.float32(left)
    unit = cs / np.float32(65536.0)
    off = np.asarray(off).astype(np.float32)
    out = np.empty((len(cell), 3), np.float32)
    for a, c in enumerate((cx, cy, cz)):
        base = lf + cs * c          # float32 * float32, then float32 + float32
        out[:, a] = base + off[:, a] * unit
    return out
