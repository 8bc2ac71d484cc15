"""The periodic buffer shell of a single-cube run: the host restatement
(synthetic.add_periodic_shell, the definition the device builder follows)
against the reference's own one-rank exchange_buffer + remove_extra_particles."""
import numpy as np
import pytest

import pyoracle as po

from asmooth_gb300 import synthetic as syn

needs_ref = pytest.mark.skipif(not po.Reference.available(), reason="reference harness not built")


def _rows(x, v):
    a = np.concatenate([x, v], axis=1)
    return a[np.lexsort(a.T[::-1])]


@needs_ref
@pytest.mark.parametrize("L,b,n", [(64.0, 8.0, 20000), (128.0, 8.0, 30000), (40.0, 6.5, 5000)])
def test_shell_matches_reference_exchange(L, b, n):
    rng = np.random.default_rng(int(L))
    x = rng.uniform(0, L, (n, 3)).astype(np.float32)
    x[:50] = rng.choice([0.0, np.float32(b), np.float32(L - b), np.nextafter(np.float32(L), 0)],
                        size=(50, 3))  # exactly on the bin thresholds and the faces
    v = rng.normal(size=(n, 3)).astype(np.float32)
    bf = np.float32(np.float32(b) / np.float32(L))
    rx, rv, rn = po.Reference().exchange_buffer(x, v, L, bf)
    cube = syn.add_periodic_shell(x, v, L, b)
    assert cube.n == len(rx) and cube.n_local == rn == n
    # interior particles first, in input order; the same shell particles, bit for bit
    assert np.array_equal(cube.x[:n], rx[:n]) and np.array_equal(cube.v[:n], rv[:n])
    assert np.array_equal(_rows(cube.x, cube.v), _rows(rx, rv))


def test_device_nfw_generator_matches_the_numpy_model():
    """nfw_cube_device (the 512^3 bench cube's generator, run here on the CPU
    device) draws the numpy generator's model: positions in [0, L), no exact
    duplicates, and the same clustering (cell-count quantiles on a 32^3 grid
    within 15% at the 99th and 99.9th percentiles)."""
    torch = pytest.importorskip("torch")
    n, L = 400_000, 128.0
    x, v = syn.nfw_cube_device(n, L, 7, n_halos=300, device="cpu")
    a = x.numpy()
    assert a.shape == (n, 3) and a.dtype == np.float32 and v.shape == (n, 3)
    assert a.min() >= 0.0 and a.max() < L
    assert np.unique(a.view(np.dtype((np.void, 12))).ravel()).size == n
    xn, _ = syn.nfw_cube(n, L, 7, n_halos=300)
    qd = np.percentile(np.histogramdd(a, bins=32)[0], [99, 99.9])
    qn = np.percentile(np.histogramdd(xn, bins=32)[0], [99, 99.9])
    assert np.all(np.abs(qd / qn - 1.0) < 0.15)
    assert isinstance(x, torch.Tensor)
