"""GPU parity tests: the CUDA path through the C ABI against the reference's own
outputs (golden fixtures) and the CPU oracle.

Bars: bit-exact rk, neighbour sets (the 33 smallest keys (d2, index)), SO-halo
marks, FOF membership and normalisation; fields within the stated tolerance of
the FP64 oracle (per-cell relative error <= 1e-5 for cells above 1e-3 of the
mean); FP64 mass totals within 1e-10 of the oracle's FP64 sum of the same
float weights."""
import os

import numpy as np
import pytest

import pyoracle as po
from helpers import DEP_TOL, rel_err_cells, set_from_key

from asmooth_gb300 import api
from asmooth_gb300 import synthetic as syn

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-5  # per-cell relative error vs FP64, cells above 1e-3 of the mean
MASS_TOL = 1e-10  # FP64 total of the deposited float weights
NTHREADS = os.cpu_count() or 1


def bits(a):
    return np.asarray(a, np.float32).view(np.int32)


def halos_of(rows):
    rows = np.asarray(rows, np.float32).reshape(-1, 5)
    return api.make_halos(rows[:, :3], rows[:, 3], rows[:, 4])


def check_mesh(mesh, m64, nc, tol=FIELD_TOL):
    """Per-cell relative error vs FP64 for cells above 1e-3 of the mean density
    (the mean of all particles' density, n + halo, over the mesh)."""
    nm = nc ** 3
    n64, h64, c64, v64 = m64[:nm], m64[nm:2 * nm], m64[2 * nm:3 * nm], m64[3 * nm:]
    n, h, c, v = mesh[:nm], mesh[nm:2 * nm], mesh[2 * nm:3 * nm], mesh[3 * nm:]
    cut = 1e-3 * float((n64 + h64).mean())
    for got, ref, dens in ((n, n64, n64), (c, c64, n64), (h, h64, h64)):
        sel = dens > cut
        if sel.any():
            err = np.abs(got[sel].astype(np.float64) - ref[sel]) / np.abs(ref[sel])
            assert err.max() <= tol
    sel = np.repeat(n64 > cut, 3)  # v against |v| + n on the same cells
    scale = (np.abs(v64) + np.repeat(n64, 3))[sel]
    assert np.all(np.abs(v.astype(np.float64)[sel] - v64[sel]) <= tol * scale)


# ---- golden fixtures (the reference's own outputs) -----------------------------------

def test_neighbor_search_golden(gpu_ctx, golden, oracle):
    g = golden
    x = g["x"]
    p = api.make_particles(x, g["v"])
    gpu_ctx.neighbor_search(p, g["left"], g["right"])
    assert np.array_equal(bits(p["rk"]), bits(g["rk"]))
    assert np.array_equal(p["x"], x) and np.array_equal(p["v"], g["v"])  # order preserved
    t33, idx33 = gpu_ctx.get_knn(len(x))
    for q, ref in zip(g["nbr_sample"], g["nbr"]):
        assert np.array_equal(set_from_key(x, int(q), t33[q], idx33[q]), ref)
    # dens: the reference's float sums in kd-tree order vs our exact fixed-point sums
    assert np.max(np.abs(p["dens"] - g["dens"]) / g["dens"]) <= FIELD_TOL
    te, ie, nbr = oracle.knn_exact(x, g["left"], g["right"], NTHREADS)
    assert np.array_equal(bits(te), bits(t33)) and np.array_equal(ie, idx33)
    _, _, d64 = oracle.dens_from_lists(x, nbr, te)
    assert np.max(np.abs(p["dens"] - d64) / d64) <= FIELD_TOL


def test_mark_halos_golden(gpu_ctx, golden):
    g = golden
    p = api.make_particles(g["x"], g["v"])
    nph, mh = gpu_ctx.mark_halo_particles(p, halos_of(g["halos"]), g["left"], g["right"])
    assert np.array_equal(p["igrp"], g["igrp_marked"])
    assert nph == g["np_halo"] and mh == g["m_halo"]


def test_mesh_golden(gpu_ctx, golden, oracle):
    g = golden
    ncs = [int(nc) for nc in g["ncs"]]
    p = api.make_particles(g["x"], g["v"], dens=g["dens"], rk=g["rk"], igrp=g["igrp_marked"])
    meshes, tot = gpu_ctx.assign_on_meshes(p, g["boxsize"], ncs, sign=-1)
    for k, nc in enumerate(ncs):
        ref = g[f"mesh{nc}"]
        _, m64, t64 = oracle.assign_on_mesh(g["x"], g["v"], g["dens"], g["rk"], g["igrp_marked"],
                                            g["boxsize"], nc, -1)
        check_mesh(meshes[k], m64, nc)
        nm = nc ** 3
        assert rel_err_cells(meshes[k][:nm], ref[:nm], ref[:nm]) <= FIELD_TOL
        assert abs(tot[k, 0] - t64[0]) <= MASS_TOL * t64[0]
        assert abs(tot[k, 1] - t64[1]) <= MASS_TOL * max(t64[1], 1.0)
        # the reference's own mass check on the float mesh
        assert abs(api.mesh_total(meshes[k], nc) - g[f"total{nc}"][0]) <= 1e-6 * g[f"total{nc}"][0]


def test_normalise_golden(gpu_ctx, golden):
    g = golden
    for nc in g["ncs"]:
        out = gpu_ctx.normalise_mesh(g[f"mesh{nc}"], int(nc), g["boxsize"])
        assert np.array_equal(bits(out), bits(g[f"norm{nc}"]))


def test_global_and_density_mesh_golden(gpu_ctx, golden, oracle):
    g = golden
    nc = int(g["ncs"][0])
    L = float(g["boxsize"])
    p = api.make_particles(g["x"], g["v"], dens=g["dens"], rk=g["rk"], igrp=g["igrp_marked"])
    mg, tg = gpu_ctx.assign_on_global_mesh(p, L, nc, -1, coords=(1, 0, 2))
    _, m64, t64 = oracle.assign_on_mesh(g["x"], g["v"], g["dens"], g["rk"], g["igrp_marked"], L, nc,
                                        -1, periodic=True, offset=(L, 0.0, 2 * L))
    check_mesh(mg, m64, nc)
    ref = g[f"global{nc}"]
    assert rel_err_cells(mg[: nc ** 3], ref[: nc ** 3], ref[: nc ** 3]) <= FIELD_TOL
    assert abs(tg[0] - t64[0]) <= MASS_TOL * t64[0]
    md = gpu_ctx.assign_on_density_mesh(p, L, nc, -1)
    ref = g[f"density{nc}"]
    assert rel_err_cells(md, ref, ref) <= FIELD_TOL


def test_fof_golden(gpu_ctx, golden):
    g = golden
    p = api.make_particles(g["x"], g["v"])
    ng = gpu_ctx.group_fof(p, g["left"], g["right"], g["ll"])
    assert ng == g["ngroup"]
    lab = p["igrp"].copy()
    assert np.array_equal(po.canonical_groups(lab), g["fof"])
    # labels 1..ng numbered by each group's smallest input index
    first = np.full(ng + 1, -1)
    for i in range(len(lab) - 1, -1, -1):
        first[lab[i]] = i
    assert lab.min() == 1 and lab.max() == ng and np.all(np.diff(first[1:]) > 0)
    nh = gpu_ctx.remove_small_groups(p, ng)
    assert nh == g["nhalo"]
    assert np.array_equal(po.canonical_groups(p["igrp"]), g["fof_halo"])


# ---- larger seeded cubes against the oracle -------------------------------------------

@pytest.mark.parametrize("name,scale", [("cfg1", 1), ("cfg2", 4)])
def test_cube_vs_oracle(gpu_ctx, oracle, name, scale):
    cube, ncs = syn.make_workload(name, scale=scale)
    x = cube.x
    p = api.make_particles(x, cube.v)
    gpu_ctx.neighbor_search(p, cube.left, cube.right)
    t33, idx33 = gpu_ctx.get_knn(cube.n)
    te, ie, nbr = oracle.knn_exact(x, cube.left, cube.right, NTHREADS)
    assert np.array_equal(bits(t33), bits(te)) and np.array_equal(idx33, ie)
    # the reference's own traversal rule (faithful port) gives the same rk
    rk_ref, dens_ref = oracle.neighbor_search(x, cube.left, cube.right)
    assert np.array_equal(bits(p["rk"]), bits(rk_ref))
    _, _, d64 = oracle.dens_from_lists(x, nbr, te)
    assert np.max(np.abs(p["dens"] - d64) / d64) <= FIELD_TOL
    assert np.max(np.abs(p["dens"] - dens_ref) / dens_ref) <= FIELD_TOL
    meshes, tot = gpu_ctx.assign_on_meshes(p, cube.boxsize, ncs, sign=-1)
    for k, nc in enumerate(ncs):
        _, m64, t64 = oracle.assign_on_mesh(x, cube.v, p["dens"], p["rk"], p["igrp"], cube.boxsize,
                                            nc, -1)
        check_mesh(meshes[k], m64, nc)
        assert abs(tot[k, 0] - t64[0]) <= MASS_TOL * t64[0]
        assert 0.999 < tot[k].sum() / cube.n_local < 1.001


def test_fof_cube_vs_oracle(gpu_ctx, oracle):
    cube, _ = syn.make_workload("cfg2", scale=4)
    p = api.make_particles(cube.x, cube.v)
    ll = np.float32(0.4)
    ng = gpu_ctx.group_fof(p, cube.left, cube.right, ll)
    lab, ng_ref = oracle.group_fof(cube.x, cube.left, cube.right, ll, exact=True)
    assert ng == ng_ref
    assert np.array_equal(po.canonical_groups(p["igrp"]), po.canonical_groups(lab))


def test_smooth_on_huge_page_host_arrays(gpu_ctx):
    """Records and meshes in asg_host_alloc blocks give the results of plain arrays."""
    cube, ncs = syn.make_workload("cfg1", scale=2)
    p1 = api.make_particles(cube.x, cube.v)
    m1, t1, _, _ = gpu_ctx.smooth(p1, cube.left, cube.right, cube.boxsize, ncs, -1)
    p2 = api.host_array(len(p1), api.PARTICLE_DTYPE)
    p2[:] = api.make_particles(cube.x, cube.v)
    m2 = [api.host_array(6 * nc ** 3) for nc in ncs]
    _, t2, _, _ = gpu_ctx.smooth(p2, cube.left, cube.right, cube.boxsize, ncs, -1, meshes=m2)
    assert p1.tobytes() == p2.tobytes()
    for a, b in zip(m1, m2):
        assert np.array_equal(bits(a), bits(b))
    assert np.array_equal(t1, t2)
    big = api.host_array(600 * 2 ** 20, np.uint8)  # past one huge page on 64 KB-page hosts
    assert big.nbytes == 600 * 2 ** 20 and big[::4096].sum() == 0


def test_smooth_pipeline_matches_staged_calls(gpu_ctx):
    cube, ncs = syn.make_workload("cfg1", scale=2)
    rng = np.random.default_rng(5)
    nh = 40
    halos = api.make_halos(cube.x[rng.choice(cube.n_local, nh)], rng.uniform(0.5, 3, nh),
                           rng.uniform(10, 1000, nh))
    p1 = api.make_particles(cube.x, cube.v)
    m1, t1, nph1, mh1 = gpu_ctx.smooth(p1, cube.left, cube.right, cube.boxsize, ncs, -1, halos)
    # staged calls on one loaded set: the same index, hence bit-identical results
    p2 = api.make_particles(cube.x, cube.v)
    gpu_ctx.load_particles(p2, cube.left, cube.right)
    gpu_ctx.run_neighbor_search()
    nph2, mh2 = gpu_ctx.run_mark_halos(halos)
    t2 = gpu_ctx.run_deposit(cube.boxsize, ncs, sign=-1)
    m2 = [gpu_ctx.copy_mesh(k, 6 * nc ** 3) for k, nc in enumerate(ncs)]
    gpu_ctx.store_particles(p2)
    assert nph1 == nph2 and mh1 == mh2
    assert p1.tobytes() == p2.tobytes()
    for a, b in zip(m1, m2):
        assert np.array_equal(bits(a), bits(b))
    assert np.array_equal(t1, t2)
    # the reference-shaped one-shot calls build their own index (own Morton grid),
    # so their sums may differ in the last bits only
    p3 = api.make_particles(cube.x, cube.v)
    gpu_ctx.neighbor_search(p3, cube.left, cube.right)
    gpu_ctx.mark_halo_particles(p3, halos, cube.left, cube.right)
    m3, t3 = gpu_ctx.assign_on_meshes(p3, cube.boxsize, ncs, sign=-1)
    assert p1.tobytes() == p3.tobytes()
    for a, b, nc in zip(m1, m3, ncs):  # each within DEP_TOL of the same FP64 sums
        n = a[: nc ** 3]
        assert rel_err_cells(b[: nc ** 3], n.astype(np.float64), n) <= 2 * DEP_TOL
    assert np.allclose(t1, t3, rtol=1e-12, atol=0)


# ---- edge cases --------------------------------------------------------------------

def test_errors_are_reported_not_faulted(gpu_ctx):
    x = np.random.default_rng(1).uniform(0, 10, (20, 3)).astype(np.float32)
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.neighbor_search(api.make_particles(x), 0.0, 10.0)
    assert e.value.status == api.ASG_ERR_FEW
    x = np.random.default_rng(2).uniform(0, 10, (100, 3)).astype(np.float32)
    x[5, 1] = np.nan
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.neighbor_search(api.make_particles(x), 0.0, 10.0)
    assert e.value.status == api.ASG_ERR_NONFINITE
    x = np.random.default_rng(3).uniform(0, 10, (100, 3)).astype(np.float32)
    x[:40] = x[0]
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.neighbor_search(api.make_particles(x), 0.0, 10.0)
    assert e.value.status == api.ASG_ERR_ZERO_RK
    p = api.make_particles(np.random.default_rng(4).uniform(0, 10, (100, 3)), rk=np.ones(100))
    with pytest.raises(api.AsmoothError) as e:
        gpu_ctx.assign_on_meshes(p, 10.0, [0])
    assert e.value.status == api.ASG_ERR_ARG
    with pytest.raises(api.AsmoothError):
        gpu_ctx.neighbor_search(api.make_particles(np.zeros((100, 3))), 1.0, 0.0)
    # the context stays usable after errors
    x = np.random.default_rng(5).uniform(0, 10, (500, 3)).astype(np.float32)
    gpu_ctx.neighbor_search(api.make_particles(x), 0.0, 10.0)


def test_lattice_ties_by_index(gpu_ctx, oracle):
    g = np.arange(10, dtype=np.float32)
    X = (np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) + 0.5).astype(np.float32)
    p = api.make_particles(X)
    gpu_ctx.neighbor_search(p, 0.0, 10.0)
    t33, idx33 = gpu_ctx.get_knn(len(X))
    te, ie, nbr = oracle.knn_exact(X, 0.0, 10.0, NTHREADS)
    assert np.array_equal(bits(t33), bits(te)) and np.array_equal(idx33, ie)
    _, _, d64 = oracle.dens_from_lists(X, nbr, te)
    assert np.max(np.abs(p["dens"] - d64) / d64) <= FIELD_TOL


@pytest.mark.parametrize("leaf", ["1", "7"])
def test_other_bucket_sizes(oracle, leaf, monkeypatch):
    """Tree buckets of 1 and 7 particles (ASG_LEAF_SIZE): the same exact
    neighbours, FOF groups and halo marks (the node boxes are built for the
    bucket size in use)."""
    monkeypatch.setenv("ASG_LEAF_SIZE", leaf)
    cube, _ = syn.make_workload("cfg1", scale=4)
    x = cube.x
    with api.Context(0) as ctx:
        p = api.make_particles(x, cube.v)
        ctx.neighbor_search(p, cube.left, cube.right)
        t33, idx33 = ctx.get_knn(cube.n)
        te, ie, _ = oracle.knn_exact(x, cube.left, cube.right, NTHREADS)
        assert np.array_equal(bits(t33), bits(te)) and np.array_equal(idx33, ie)
        q = api.make_particles(x)
        ng = ctx.group_fof(q, cube.left, cube.right, np.float32(0.4))
        lab, ng_ref = oracle.group_fof(x, cube.left, cube.right, np.float32(0.4), exact=True)
        assert ng == ng_ref
        assert np.array_equal(po.canonical_groups(q["igrp"]), po.canonical_groups(lab))


def test_empty_halo_list_and_small_sets(gpu_ctx):
    x = np.random.default_rng(9).uniform(0, 10, (33, 3)).astype(np.float32)
    p = api.make_particles(x)
    gpu_ctx.neighbor_search(p, 0.0, 10.0)  # exactly 33 particles: rk = farthest
    d2max = max(float(((x - x[i]) ** 2).sum(1).max()) for i in range(1))
    assert abs(p["rk"][0] ** 2 - d2max) <= 1e-5 * d2max
    assert gpu_ctx.mark_halo_particles(p, api.make_halos(np.zeros((0, 3)), [], []), 0.0, 10.0) == (0, 0.0)


def test_deep_ties_at_33rd(gpu_ctx, oracle):
    """Queries whose 33rd key sits behind many exact ties (KNeighbors::push in
    k_neighbors.h:25-35 resolves any multiplicity): a particle with two closer
    particles and 30 more at exactly d2 = 25 (integer offsets (5,0,0), (3,4,0)
    and their permutations and signs), so the 33rd key is the 30th smallest
    tied index.  Several such clusters, indices shuffled, far apart."""
    shell = set()
    for a in (5, 3, 4, 0):
        for b in (5, 3, 4, 0):
            for c in (5, 3, 4, 0):
                if a * a + b * b + c * c == 25:
                    for sx in (1, -1):
                        for sy in (1, -1):
                            for sz in (1, -1):
                                shell.add((sx * a, sy * b, sz * c))
    shell = np.array(sorted(shell), np.float32)
    assert len(shell) == 30
    pts = []
    for k in range(12):
        c = np.float32([40.0 * (k % 3), 40.0 * ((k // 3) % 2), 40.0 * (k // 6)]) + 20.0
        pts += [c, c + np.float32([1, 0, 0]), c + np.float32([0, 2, 0])]
        pts += list(c + shell)
    X = np.array(pts, np.float32)
    X = X[np.random.default_rng(4).permutation(len(X))]
    p = api.make_particles(X)
    gpu_ctx.neighbor_search(p, 0.0, 140.0)
    t33, idx33 = gpu_ctx.get_knn(len(X))
    te, ie, nbr = oracle.knn_exact(X, 0.0, 140.0, NTHREADS)
    assert np.array_equal(bits(t33), bits(te)) and np.array_equal(idx33, ie)
    assert np.sum(t33 == 25.0) >= 12  # the cluster centres' 33rd key is behind 30 ties
    _, _, d64 = oracle.dens_from_lists(X, nbr, te)
    assert np.max(np.abs(p["dens"] - d64) / d64) <= FIELD_TOL
    # the same without get_knn: the pipeline's own tie pass (flagged queries only)
    p2 = api.make_particles(X)
    gpu_ctx.neighbor_search(p2, 0.0, 140.0)
    assert p.tobytes() == p2.tobytes()


@pytest.mark.parametrize("periodic", [False, True])
def test_deposit_tile_order_changes_no_bit(oracle, periodic, monkeypatch):
    """The persistent deposit takes the tiles of all meshes in a Morton order
    (ASG_DEPOSIT_ORDER=tile: tile order).  The order only changes when each
    tile is summed, not how, so meshes and FP64 totals are bit-identical."""
    cube, ncs = syn.make_workload("cfg2", scale=4)
    out = {}
    for order in ("tile", "morton"):
        monkeypatch.setenv("ASG_DEPOSIT_ORDER", order)
        with api.Context(0) as ctx:
            p = api.make_particles(cube.x, cube.v)
            ctx.neighbor_search(p, cube.left, cube.right)
            out[order] = ctx.assign_on_meshes(p, cube.boxsize, ncs, sign=-1, periodic=periodic)
    (m0, t0), (m1, t1) = out["tile"], out["morton"]
    for a, b in zip(m0, m1):
        assert np.array_equal(bits(a), bits(b))
    assert np.array_equal(t0, t1)
