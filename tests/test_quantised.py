"""Mixed-precision positions (int32 cell index + uint16 offsets): the host
decode definition and what quantisation does to the neighbour search, on the
CPU oracle."""
import os

import numpy as np

from asmooth_gb300 import quantised as qz
from asmooth_gb300 import synthetic as syn

NTHREADS = os.cpu_count() or 1


def test_decode_is_exact_and_inside_the_cell():
    cube, _ = syn.make_workload("cfg2", scale=8)
    cell, off, grid = syn.quantise_positions(cube)
    assert cell.dtype == np.int32 and off.dtype == np.uint16 and off.shape == (cube.n, 3)
    assert grid == 20  # (side 64 + 2 x 8-unit shell) / 4-unit cells
    assert cell.min() >= 0 and cell.max() < grid ** 3
    xq = qz.dequantise(cell, off, grid, cube.left)
    # every decoded coordinate is a multiple of 2^-14: float32 holds it exactly
    assert np.all(np.mod(xq.astype(np.float64) * 16384.0, 1.0) == 0.0)
    # truncation toward the cell's lower corner, by less than one offset unit
    d = cube.x.astype(np.float64) - xq.astype(np.float64)
    assert d.min() >= 0.0 and d.max() < 4.0 / 65536.0


def test_decode_order_of_operations():
    # (left + cs*cx) + off*unit in float32, for a cell size whose unit is not a power of 2
    cs, left, grid = 3.0, -8.0, 7
    cell = np.array([0, 1, grid, grid * grid, grid ** 3 - 1], np.int32)
    off = np.array([[0, 0, 0], [1, 2, 3], [65535, 0, 7], [12345, 54321, 1], [65535] * 3], np.uint16)
    xq = qz.dequantise(cell, off, grid, left, cs)
    unit = np.float32(cs) / np.float32(65536.0)
    cx = cell % grid
    want = (np.float32(left) + np.float32(cs) * cx.astype(np.float32)) + off[:, 0].astype(np.float32) * unit
    assert np.array_equal(xq[:, 0], want.astype(np.float32))
    assert xq[1, 0] == np.float32(np.float32(-5.0) + np.float32(unit))


def test_grid_covers_the_cube():
    for left, right, cs in ((-8.0, 520.0, 4.0), (-8.0, 1032.0, 4.0), (0.0, 10.0, 3.0)):
        g = qz.grid_size(left, right, cs)
        assert np.float32(left) + np.float32(cs) * np.float32(g) >= np.float32(right)
        assert np.float32(left) + np.float32(cs) * np.float32(g - 1) < np.float32(right)


def test_neighbour_sets_under_quantisation(oracle):
    """The mixed form's neighbour sets are exact for its decoded positions; this
    states how far they move from the FP32 positions' sets (reported, not a
    parity bar): >= 99% identical 33-sets; h moves by at most the largest
    change of a pair distance, 2*sqrt(3)*4/65536, median relative <= 1e-4."""
    cube, _ = syn.make_workload("cfg2", scale=8)
    cell, off, grid = syn.quantise_positions(cube)
    xq = qz.dequantise(cell, off, grid, cube.left)
    te, _, nbr = oracle.knn_exact(cube.x, cube.left, cube.right, NTHREADS)
    tq, _, nbq = oracle.knn_exact(xq, cube.left, cube.right, NTHREADS)
    same = np.mean([np.array_equal(np.sort(a), np.sort(b)) for a, b in zip(nbr, nbq)])
    h, hq = np.sqrt(te.astype(np.float64)), np.sqrt(tq.astype(np.float64))
    assert same >= 0.99
    assert np.all(np.abs(hq - h) <= 2 * np.sqrt(3) * 4.0 / 65536 + 1e-6 * h)
    assert np.median(np.abs(hq - h) / h) <= 1e-4
