"""GPU tests of the device-built periodic shell (single-cube run): the same
particles, float positions and order as the host definition
(synthetic.add_periodic_shell, whose particle set equals the reference's
one-rank exchange_buffer + remove_extra_particles, tests/test_shell.py), and
the same path results as loading that host-built set."""
import numpy as np
import pytest

from asmooth_gb300 import api
from asmooth_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu


def _interior(name, scale):
    cube, ncs = syn.make_workload(name, scale=scale)
    n = cube.n_local
    return cube, ncs, cube.x[:n].copy(), cube.v[:n].copy()


def _bf(cube):
    return np.float32(np.float32(cube.left * -1.0) / np.float32(cube.boxsize))


def test_device_shell_equals_host_shell(gpu_ctx):
    cube, _, x, v = _interior("cfg1", 2)
    p = api.make_particles(x, v)
    nw, nl = gpu_ctx.load_periodic_cube(p, cube.boxsize, _bf(cube))
    assert (nw, nl) == (cube.n, cube.n_local)
    q = np.zeros(nw, api.PARTICLE_DTYPE)
    gpu_ctx.store_particles(q)
    assert np.array_equal(q["x"], cube.x) and np.array_equal(q["v"], cube.v)


def test_device_shell_path_results(gpu_ctx):
    cube, ncs, x, v = _interior("cfg2", 4)
    p = api.make_particles(x, v)
    nw, _ = gpu_ctx.load_periodic_cube(p, cube.boxsize, _bf(cube))
    gpu_ctx.run_neighbor_search()
    tot1 = gpu_ctx.run_deposit(cube.boxsize, ncs, sign=-1)
    m1 = [gpu_ctx.copy_mesh(k, 6 * nc ** 3) for k, nc in enumerate(ncs)]
    q = np.zeros(nw, api.PARTICLE_DTYPE)
    gpu_ctx.store_particles(q)
    # the host-built set through the plain loader: bit-identical results
    r = api.make_particles(cube.x, cube.v)
    gpu_ctx.load_particles(r, cube.left, cube.right)
    gpu_ctx.run_neighbor_search()
    tot2 = gpu_ctx.run_deposit(cube.boxsize, ncs, sign=-1)
    gpu_ctx.store_particles(r)
    assert np.array_equal(q["rk"].view(np.int32), r["rk"].view(np.int32))
    assert np.array_equal(q["dens"].view(np.int32), r["dens"].view(np.int32))
    for k, nc in enumerate(ncs):
        assert np.array_equal(m1[k], gpu_ctx.copy_mesh(k, 6 * nc ** 3))
    assert np.array_equal(tot1, tot2)


def test_device_shell_from_device_arrays(gpu_ctx):
    torch = pytest.importorskip("torch")
    cube, _, x, v = _interior("cfg1", 4)
    xd, vd = torch.from_numpy(x).cuda(), torch.from_numpy(v).cuda()
    nw, nl = gpu_ctx.load_periodic_cube_device(xd.data_ptr(), len(x), cube.boxsize, _bf(cube),
                                               v_ptr=vd.data_ptr())
    torch.cuda.synchronize()
    assert (nw, nl) == (cube.n, cube.n_local)
    q = np.zeros(nw, api.PARTICLE_DTYPE)
    gpu_ctx.store_particles(q)
    assert np.array_equal(q["x"], cube.x) and np.array_equal(q["v"], cube.v)


def test_device_shell_bad_arguments(gpu_ctx):
    p = api.make_particles(np.random.default_rng(0).uniform(0, 10, (100, 3)))
    for L, bf in ((10.0, 0.0), (10.0, 0.5), (0.0, 0.1), (-1.0, 0.1)):
        with pytest.raises(api.AsmoothError) as e:
            gpu_ctx.load_periodic_cube(p, L, bf)
        assert e.value.status == api.ASG_ERR_ARG
    gpu_ctx.load_periodic_cube(p, 10.0, 0.2)  # the context stays usable
