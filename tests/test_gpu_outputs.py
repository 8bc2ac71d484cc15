"""GPU tests of the outputs through the C ABI: the mesh files of
write_mesh_separate and the FOF halo catalogue of write_fof_halos, bit for bit
against the oracle (whose formats and values are pinned to the reference's own
files by tests/test_writers.py)."""
import os
import struct

import numpy as np
import pytest

import pyoracle as po

from asmooth_gb300 import api
from asmooth_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _expected_files(oracle, raw, nc, boxsize):
    norm = oracle.normalise_mesh(raw, nc, boxsize)
    nm = nc ** 3
    head = struct.pack("<i", nc)
    return {"n": head + norm[:nm].tobytes(), "h": head + norm[nm:2 * nm].tobytes(),
            "c": head + norm[2 * nm:3 * nm].tobytes(), "vel": head + norm[3 * nm:].tobytes()}


def test_write_mesh_separate_files(gpu_ctx, oracle, tmp_path):
    cube, ncs = syn.make_workload("cfg1", scale=4)
    p = api.make_particles(cube.x, cube.v)
    gpu_ctx.neighbor_search(p, cube.left, cube.right)
    nc = ncs[0]
    raw, _ = gpu_ctx.assign_on_mesh(p, cube.boxsize, nc, sign=-1)
    want = _expected_files(oracle, raw, nc, cube.boxsize)
    base = str(tmp_path / "so" / "nc") + f"{nc}/0.000"
    os.makedirs(os.path.dirname(base))
    m = raw.copy()
    gpu_ctx.write_mesh_separate(base, 2, m, nc, cube.boxsize)
    for ch, b in want.items():
        assert open(f"{base}{ch}2.dat", "rb").read() == b
    assert m.tobytes() == oracle.normalise_mesh(raw, nc, cube.boxsize).tobytes()  # in place


def test_write_mesh_device_files(gpu_ctx, oracle, tmp_path):
    cube, ncs = syn.make_workload("cfg1", scale=4)
    x = cube.x
    p = api.make_particles(x, cube.v)
    gpu_ctx.load_particles(p, cube.left, cube.right)
    gpu_ctx.run_neighbor_search()
    gpu_ctx.run_deposit(cube.boxsize, ncs, sign=-1)
    for k, nc in enumerate(ncs):
        raw = gpu_ctx.copy_mesh(k, 6 * nc ** 3)
        want = _expected_files(oracle, raw, nc, cube.boxsize)
        base = str(tmp_path) + f"/k{k}_"
        gpu_ctx.write_mesh_device(k, base, 0)
        for ch, b in want.items():
            assert open(f"{base}{ch}0.dat", "rb").read() == b


def test_fof_catalogue_vs_oracle(gpu_ctx, oracle, tmp_path):
    cube, _ = syn.make_workload("cfg2", scale=4)
    p = api.make_particles(cube.x, cube.v)
    ng = gpu_ctx.group_fof(p, cube.left, cube.right, np.float32(0.4))
    nh = gpu_ctx.remove_small_groups(p, ng)
    want = oracle.fof_halos(cube.x, cube.v, p["igrp"], nh, cube.boxsize)
    assert len(want) > 10
    got = gpu_ctx.fof_halos(p, nh, cube.boxsize)
    assert got.tobytes() == want.tobytes()
    fn = str(tmp_path / "fof0.dat")
    gpu_ctx.write_fof_halos(fn, p, nh, cube.boxsize)
    b = open(fn, "rb").read()
    assert b == struct.pack("<ii", len(want), 28) + want.tobytes() + struct.pack("<i", len(want))
    # staged: the loaded set's labels, summed in load order
    gpu_ctx.load_particles(p, cube.left, cube.right)
    assert gpu_ctx.run_fof_halos(nh, cube.boxsize).tobytes() == want.tobytes()


def test_fof_catalogue_array_order(gpu_ctx, oracle):
    """Float sums follow the caller's array order: a permuted array gives the
    oracle's result for that permutation."""
    cube, _ = syn.make_workload("cfg1", scale=2)
    p = api.make_particles(cube.x, cube.v)
    ng = gpu_ctx.group_fof(p, cube.left, cube.right, np.float32(0.4))
    nh = gpu_ctx.remove_small_groups(p, ng)
    perm = np.random.default_rng(1).permutation(len(p))
    q = p[perm].copy()
    want = oracle.fof_halos(q["x"], q["v"], q["igrp"], nh, cube.boxsize)
    assert gpu_ctx.fof_halos(q, nh, cube.boxsize).tobytes() == want.tobytes()


def test_writer_io_error(gpu_ctx, tmp_path):
    m = np.zeros(6 * 4 ** 3, np.float32)
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.write_mesh_separate(str(tmp_path / "missing" / "x"), 0, m, 4, 10.0)
    assert e.value.status == api.ASG_ERR_IO
    p = api.make_particles(np.zeros((40, 3), np.float32))
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.write_fof_halos(str(tmp_path / "missing" / "f.dat"), p, 0, 10.0)
    assert e.value.status == api.ASG_ERR_IO
