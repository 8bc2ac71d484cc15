"""Output formats on the CPU: the library's host writer against the
reference's own (oracle/_ref), and the oracle's FOF catalogue and the mesh
file layout pinned to the reference's files."""
import os
import struct

import numpy as np
import pytest

import pyoracle as po

from asmooth_gb300 import api
from asmooth_gb300 import synthetic as syn

needs_ref = pytest.mark.skipif(not po.Reference.available(), reason="reference harness not built")


def _mesh(nc, seed=3):
    rng = np.random.default_rng(seed)
    m = rng.uniform(0, 5, 6 * nc ** 3).astype(np.float32)
    m[: nc ** 3][rng.random(nc ** 3) < 0.2] = 0.0  # empty cells take the n == 0 branch
    return m


@needs_ref
def test_write_mesh_bytes_match_reference(tmp_path):
    nc, L = 8, 128.0
    m = _mesh(nc)
    ours, ref = str(tmp_path / "ours.dat"), str(tmp_path / "ref.dat")
    api.write_mesh(ours, m, nc, L)
    po.Reference().write_mesh(ref, m, nc, L)
    assert open(ours, "rb").read() == open(ref, "rb").read()
    b = open(ours, "rb").read()
    assert struct.unpack("<iif", b[:12]) == (nc, 6, L) and len(b) == 12 + 24 * nc ** 3


@needs_ref
def test_mesh_separate_layout_pinned(tmp_path, oracle):
    """The reference's four files are `int nc` + the normalised channels; the
    GPU writer tests build their expected bytes this way."""
    nc, L = 8, 128.0
    m = _mesh(nc)
    base = str(tmp_path / "so") + "/"
    os.makedirs(base)
    po.Reference().write_mesh_separate(base, 5, m, nc, L)
    norm = oracle.normalise_mesh(m, nc, L)
    nm = nc ** 3
    head = struct.pack("<i", nc)
    want = {"n": norm[:nm], "h": norm[nm:2 * nm], "c": norm[2 * nm:3 * nm], "vel": norm[3 * nm:]}
    for ch, arr in want.items():
        assert open(f"{base}{ch}5.dat", "rb").read() == head + arr.tobytes()


@needs_ref
def test_fof_catalogue_oracle_matches_reference(tmp_path, oracle):
    cube, _ = syn.make_workload("cfg2", scale=4)
    lab, ng = oracle.group_fof(cube.x, cube.left, cube.right, np.float32(0.4))
    lab, nh = oracle.remove_small_groups(lab, ng)
    rec = oracle.fof_halos(cube.x, cube.v, lab, nh, cube.boxsize)
    fn = str(tmp_path / "fof0.dat")
    po.Reference().write_fof_halos(fn, cube.x, cube.v, lab, nh, cube.boxsize)
    b = open(fn, "rb").read()
    nl, size = struct.unpack("<ii", b[:8])
    assert size == 28 and nl == len(rec) and 0 < nl <= nh
    assert b[8:8 + 28 * nl] == rec.tobytes()
    assert struct.unpack("<i", b[8 + 28 * nl:]) == (nl,)


def test_write_mesh_rejects_bad_input(tmp_path):
    with pytest.raises(ValueError):
        api.write_mesh(str(tmp_path / "x.dat"), np.zeros(10, np.float32), 8, 1.0)
    with pytest.raises(api.AsmoothError) as e:
        api.write_mesh(str(tmp_path / "missing" / "x.dat"), _mesh(4), 4, 1.0)
    assert e.value.status == api.ASG_ERR_IO
