"""GPU tests of the particle-file decode (xv conversion, zip count-prefix
expansion) against the oracle's restatement of read_pm_file_zip (pinned to
the reference's reader in tests/test_decode.py), and the decoded set fed to
the device-built periodic shell."""
import os

import numpy as np
import pytest

from test_decode import SHIFT, zip_case

from asmooth_gb300 import api
from asmooth_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def test_zip_decode_vs_oracle(gpu_ctx, oracle, tmp_path):
    fb, x, v, order = zip_case(tmp_path)
    n, L = gpu_ctx.read_pm_file_zip(fb, "6.000", 0, 16, 4, SHIFT)
    xo, vo, Lo = oracle.decode_zip(fb, "6.000", 0, 16, 4, SHIFT)
    assert n == len(xo) and L == Lo
    p = gpu_ctx.copy_decoded(n)
    assert np.array_equal(p["x"], xo) and np.array_equal(p["v"], vo)
    assert not p["rk"].any() and not p["dens"].any() and not p["igrp"].any()


def test_xv_decode(gpu_ctx, tmp_path):
    rng = np.random.default_rng(2)
    x = rng.uniform(0, 64, (7000, 3)).astype(np.float32)
    v = rng.normal(size=(7000, 3)).astype(np.float32)
    fb = str(tmp_path / "node")
    os.makedirs(fb + "3")
    syn.write_xv(syn.xv_path(fb, "0.000", 3), x, v)
    n = gpu_ctx.read_pm_file_xv(fb, "0.000", 3, SHIFT)
    p = gpu_ctx.copy_decoded(n)
    assert np.array_equal(p["x"], x - np.float32(SHIFT)) and np.array_equal(p["v"], v)
    n2 = gpu_ctx.decode_xv(np.concatenate([x, v], axis=1))
    assert np.array_equal(gpu_ctx.copy_decoded(n2)["x"], x)


def test_decoded_periodic_equals_host_records(gpu_ctx, tmp_path):
    # a whole box decoded from zip files, then the shell on the device
    rng = np.random.default_rng(3)
    L, nc, scale = 64.0, 16, 4
    x = rng.uniform(0, L, (30000, 3)).astype(np.float32)
    v = rng.normal(size=(30000, 3)).astype(np.float32)
    fb = str(tmp_path / "node")
    syn.write_zip(fb, "3.000", 0, x, v, nc, scale, np.float32(50.0))
    n, Lz = gpu_ctx.read_pm_file_zip(fb, "3.000", 0, nc, scale)
    p = gpu_ctx.copy_decoded(n)
    bf = np.float32(np.float32(8.0) / np.float32(Lz))
    nw1, nl1 = gpu_ctx.load_decoded_periodic(Lz, bf)
    q1 = np.zeros(nw1, api.PARTICLE_DTYPE)
    gpu_ctx.store_particles(q1)
    nw2, nl2 = gpu_ctx.load_periodic_cube(p, Lz, bf)
    q2 = np.zeros(nw2, api.PARTICLE_DTYPE)
    gpu_ctx.store_particles(q2)
    assert (nw1, nl1) == (nw2, nl2) and q1.tobytes() == q2.tobytes()
    cube = syn.add_periodic_shell(p["x"], p["v"], Lz, 8.0)
    assert np.array_equal(q1["x"], cube.x)


def test_decode_errors(gpu_ctx, tmp_path):
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.read_pm_file_zip(str(tmp_path / "none"), "0.000", 0, 8, 4)
    assert e.value.status == api.ASG_ERR_IO
    # counts that do not sum to np_local
    z2 = np.full(8 ** 3, 1, np.uint8)
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.decode_zip(np.zeros(3 * 500, np.uint8), np.zeros(3 * 500, np.int16), z2,
                           np.zeros(0, np.int32), 500, 8, 4, 1.0)
    assert e.value.status == api.ASG_ERR_ARG
    # a 255-cell without its zip3 count
    z2[0] = 255
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.decode_zip(np.zeros(3 * 511, np.uint8), np.zeros(3 * 511, np.int16), z2,
                           np.zeros(0, np.int32), 511, 8, 4, 1.0)
    assert e.value.status == api.ASG_ERR_ARG
    gpu_ctx.decode_xv(np.ones((40, 6), np.float32))  # the context stays usable
