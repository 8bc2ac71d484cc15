"""GPU test of asg_neighbor_search_noalloc, the entry point for callers that
cannot allocate device memory (for example a host code whose memory manager
owns the whole GPU and lends libraries only its own buffers).

It is called through the C ABI on the caller's device buffers, twice in a row
(the fixed scratch keeps the first call's contents), and must give the same rk
and dens as the allocating neighbour search on the same particles: rk bit for
bit, dens within the 1e-5 relative tolerance of the other parity tests.  The
second call adds onto a non-zero dens, as the reference's `dens +=` does, and
must leave the device's free memory unchanged.  This file is collected last
so that a run stopping at the first failure has already run every other
test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5


def test_noalloc_matches_allocating_search():
    torch = pytest.importorskip("torch")
    from asmooth_gb300 import _lib, api
    from asmooth_gb300 import build as B
    from asmooth_gb300 import synthetic as syn

    B.build()
    lib = _lib.load()
    cube, _ = syn.make_workload("cfg1", scale=4)  # 13840 particles with the shell
    n = cube.n
    assert n <= 32768
    x_d = torch.from_numpy(cube.x).cuda()

    # the existing, allocating entry point on the same device arrays
    with api.Context(0) as ctx:
        ctx.load_particles_device(x_d.data_ptr(), n, cube.left, cube.right)
        ctx.run_neighbor_search()
        rk_ref = torch.empty(n, dtype=torch.float32, device="cuda")
        dens_ref = torch.empty(n, dtype=torch.float32, device="cuda")
        ctx.store_fields_device(rk_ptr=rk_ref.data_ptr(), dens_ptr=dens_ref.data_ptr())
    torch.cuda.synchronize()
    rk_ref, dens_ref = rk_ref.cpu().numpy(), dens_ref.cpu().numpy()

    # preparing call: loads the module (places the scratch) and finds its address
    assert lib.asg_neighbor_search_noalloc(None, 0, 0.0, 0.0, None, None, None) == 0

    # every buffer of both calls exists before the first one runs
    dens0 = np.random.default_rng(3).uniform(0.5, 2.0, n).astype(np.float32)
    bufs = [(torch.full((n,), -1.0, dtype=torch.float32, device="cuda"),
             torch.from_numpy(d).cuda()) for d in (np.zeros(n, np.float32), dens0)]
    torch.cuda.synchronize()
    free = []
    for (rk, dens), d_in in zip(bufs, (np.zeros(n, np.float32), dens0)):
        # the second call runs on the scratch the first one left behind
        rc = lib.asg_neighbor_search_noalloc(C.c_void_p(x_d.data_ptr()), n, cube.left, cube.right,
                                             C.c_void_p(rk.data_ptr()), C.c_void_p(dens.data_ptr()),
                                             None)
        assert rc == 0, lib.asg_strerror(rc)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        rk_h, dens_h = rk.cpu().numpy(), dens.cpu().numpy()
        assert np.array_equal(rk_h.view(np.int32), rk_ref.view(np.int32))
        want = d_in.astype(np.float64) + dens_ref  # dens is added to, not overwritten
        assert np.max(np.abs(dens_h - want) / want) <= FIELD_TOL
    # the call allocated nothing on the device
    assert free[1] == free[0]

    # inputs beyond the fixed scratch are refused with a clear status
    big = torch.zeros((32769, 3), dtype=torch.float32, device="cuda")
    out = torch.zeros(32769, dtype=torch.float32, device="cuda")
    rc = lib.asg_neighbor_search_noalloc(C.c_void_p(big.data_ptr()), 32769, 0.0, 1.0,
                                         C.c_void_p(out.data_ptr()), C.c_void_p(out.data_ptr()), None)
    assert rc == api.ASG_ERR_NOALLOC_LIMIT
    assert b"scratch" in lib.asg_strerror(rc)
