"""GPU tests of the mixed-precision form (int32 cell index + uint16 offsets,
decoded on the device, FP32 distances and weights).

Bars: on the decoded positions the mixed form gives the plain form's results
bit for bit (same FP32 path), hence the oracle's neighbour sets and rk exactly
and fields within the plain form's tolerance; against the original FP32
positions it stays within the quantisation bounds."""
import os

import numpy as np
import pytest

from asmooth_gb300 import api
from asmooth_gb300 import quantised as qz
from asmooth_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5
NTHREADS = os.cpu_count() or 1


def bits(a):
    return np.asarray(a, np.float32).view(np.int32)


def test_mixed_equals_plain_on_decoded_positions(gpu_ctx):
    cube, ncs = syn.make_workload("cfg2", scale=4)
    cell, off, grid = syn.quantise_positions(cube)
    xq = qz.dequantise(cell, off, grid, cube.left)
    rk, dens, m1, t1 = gpu_ctx.smooth_quantised(cell, off, cube.v, cube.left, cube.right, 4.0, grid,
                                                cube.boxsize, ncs, -1)
    p = api.make_particles(xq, cube.v)
    m2, t2, _, _ = gpu_ctx.smooth(p, cube.left, cube.right, cube.boxsize, ncs, -1)
    assert np.array_equal(bits(rk), bits(p["rk"]))
    assert np.array_equal(bits(dens), bits(p["dens"]))
    for a, b in zip(m1, m2):
        assert np.array_equal(bits(a), bits(b))
    assert np.array_equal(t1, t2)


def test_mixed_staged_vs_oracle(gpu_ctx, oracle):
    cube, _ = syn.make_workload("cfg1", scale=2)
    cell, off, grid = syn.quantise_positions(cube)
    xq = qz.dequantise(cell, off, grid, cube.left)
    gpu_ctx.load_particles_quantised(cell, off, cube.v, cube.left, cube.right, 4.0, grid)
    gpu_ctx.run_neighbor_search()
    t33, idx33 = gpu_ctx.get_knn(cube.n)
    te, ie, nbr = oracle.knn_exact(xq, cube.left, cube.right, NTHREADS)
    assert np.array_equal(bits(t33), bits(te)) and np.array_equal(idx33, ie)
    p = api.make_particles(xq, cube.v)
    gpu_ctx.store_particles(p)
    assert np.array_equal(p["x"], xq)  # the decoded positions come back in input order
    rk_ref, _ = oracle.neighbor_search(xq, cube.left, cube.right)
    assert np.array_equal(bits(p["rk"]), bits(rk_ref))
    _, _, d64 = oracle.dens_from_lists(xq, nbr, te)
    assert np.max(np.abs(p["dens"] - d64) / d64) <= FIELD_TOL


def test_mixed_vs_fp32_positions(gpu_ctx):
    """Against the unquantised positions.  Each coordinate moves by less than
    4/65536, so every pair distance, and with it the 33rd-neighbour distance,
    moves by at most 2*sqrt(3)*4/65536: |h_mixed - h| stays within that (plus
    float rounding), median relative change <= 1e-4; FP64 mass totals within
    1e-6 relative."""
    cube, ncs = syn.make_workload("cfg2", scale=4)
    cell, off, grid = syn.quantise_positions(cube)
    rk, dens, _, tq = gpu_ctx.smooth_quantised(cell, off, cube.v, cube.left, cube.right, 4.0, grid,
                                               cube.boxsize, ncs, -1)
    p = api.make_particles(cube.x, cube.v)
    _, tp, _, _ = gpu_ctx.smooth(p, cube.left, cube.right, cube.boxsize, ncs, -1)
    h = p["rk"].astype(np.float64)
    dh = np.abs(rk.astype(np.float64) - h)
    assert np.all(dh <= 2 * np.sqrt(3) * 4.0 / 65536 + 4 * np.spacing(p["rk"]).astype(np.float64))
    assert np.median(dh / h) <= 1e-4
    assert np.all(np.abs(tq - tp) <= 1e-6 * np.abs(tp) + 1e-9)


def test_mixed_bad_cell_is_an_argument_error(gpu_ctx):
    cube, _ = syn.make_workload("cfg1", scale=4)
    cell, off, grid = syn.quantise_positions(cube)
    bad = cell.copy()
    bad[7] = grid ** 3
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.load_particles_quantised(bad, off, cube.v, cube.left, cube.right, 4.0, grid)
    assert e.value.status == api.ASG_ERR_ARG
    with pytest.raises(api.AsmoothError):  # grid too small for [left, right)
        gpu_ctx.load_particles_quantised(cell, off, cube.v, cube.left, cube.right, 4.0, 3)
    # the context stays usable
    gpu_ctx.load_particles_quantised(cell, off, cube.v, cube.left, cube.right, 4.0, grid)
    gpu_ctx.run_neighbor_search()
