"""Particle files on the CPU: the zip writer and the oracle's decode of
read_pm_file_zip / read_pm_file_xv pinned to the reference's own readers."""
import os

import numpy as np
import pytest

import pyoracle as po

from asmooth_gb300 import synthetic as syn

needs_ref = pytest.mark.skipif(not po.Reference.available(), reason="reference harness not built")

SHIFT = (0.5, 0.25, 0.0)


def zip_case(tmp_path, nc=16, scale=4, clump=600, seed=0):
    """Particles inside the zip grid (after the shift), with a clump whose
    fine cell holds more than 255 particles (a zip3 count)."""
    rng = np.random.default_rng(seed)
    L = nc * scale
    x = rng.uniform(0, L, (20000, 3)).astype(np.float32) - np.float32(SHIFT)
    x = np.concatenate([x, np.float32(10.0) + rng.uniform(0, 0.5, (clump, 3)).astype(np.float32)])
    x = np.clip(x, -np.float32(SHIFT), L - np.float32(SHIFT) - 1e-3).astype(np.float32)
    v = rng.normal(0, 3, x.shape).astype(np.float32)
    fb = str(tmp_path / "node")
    order = syn.write_zip(fb, "6.000", 0, x, v, nc, scale, np.float32(100.0), SHIFT)
    return fb, x, v, order


@needs_ref
def test_zip_decode_matches_reference(tmp_path, oracle):
    fb, x, v, order = zip_case(tmp_path)
    assert os.path.getsize(syn.zip_paths(fb, "6.000", 0)[3]) > 0  # some cell needs zip3
    xo, vo, Lo = oracle.decode_zip(fb, "6.000", 0, 16, 4, SHIFT)
    xr, vr, Lr = po.Reference().read_pm_file_zip(fb, "6.000", 0, 16, 4, len(x) + 8, SHIFT)
    assert np.array_equal(xo, xr) and np.array_equal(vo, vr) and Lo == Lr == 64.0
    # the writer's quantisation: within 1/256 of a cell and 1/v_r2i
    assert np.abs(xo - x[order]).max() <= 4.0 / 256.0 + 1e-5
    assert np.abs(vo - v[order]).max() <= 0.5 / 100.0 + 1e-6


@needs_ref
def test_xv_read_matches_reference(tmp_path):
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 64, (5000, 3)).astype(np.float32)
    v = rng.normal(size=(5000, 3)).astype(np.float32)
    fb = str(tmp_path / "node")
    os.makedirs(fb + "0")
    syn.write_xv(syn.xv_path(fb, "1.500", 0), x, v)
    xr, vr = po.Reference().read_pm_file_xv(fb, "1.500", 0, 5008, SHIFT)
    assert np.array_equal(xr, x - np.float32(SHIFT)) and np.array_equal(vr, v)
