"""GPU deposit on adversarial inputs: particles exactly on cell and 8-cell tile
edges and next to them, supports that end exactly on edges, particles past the
box faces (clipping), halo and non-halo particles under both signs, in the
plain (coarse_mesh.cpp:45-127), periodic (global_mesh.cpp:25-123) and
density-only (coarse_mesh.cpp:212-269) deposits.

The library evaluates each cell's 1-D tent integral more accurately than the
reference's float ker_integ (coarse_mesh.cpp:10-22, 80-90): cell edges as
fma(i, dx, -x) * hinv and cancellation-free forms of the integral; a cell's
weight is the product of the three, formed on the tensor cores.  The oracle
restates the 1-D weights in C (lib_weight) and sums the products in FP64.
Three checks, all through the C ABI:
  * disjoint supports: the particles are split into batches whose cell boxes
    do not overlap, so every cell receives at most one weight, which must match
    the oracle's to DEP_TOL relative in n, c and halo, v within DEP_TOL of
    |v| + n;
  * the whole set at once: the same bars on every cell, and the FP64 mass
    totals within 1e-12 of the FP64 sums of the weights;
  * accuracy: every channel within 1e-5 of the FP64 restatement (cells above
    1e-3 of the mean density), the bar the reference's own float weights miss
    on these inputs."""
import numpy as np
import pytest

from helpers import DEP_TOL, EDGE_L as L, EDGE_NCS as NCS, edge_inputs, field_errors

from asmooth_gb300 import api

pytestmark = pytest.mark.gpu

TOTAL_TOL = 1e-12
FIELD_TOL = 1e-5


def bits(a):
    return np.asarray(a, np.float32).view(np.int32)


def axis_cells(x, h, nc, periodic):
    """A superset of the cells each particle touches along one axis, as a
    boolean (n, nc) array (one cell of margin on each side; wrapped when periodic)."""
    f = (x.astype(np.float64) / L) * nc
    w = (h.astype(np.float64) / L) * nc
    lo = np.floor(f - w).astype(np.int64) - 1
    hi = np.floor(f + w).astype(np.int64) + 2
    cells = np.zeros((x.size, nc), bool)
    for i in range(x.size):
        r = np.arange(lo[i], hi[i])
        r = np.mod(r, nc) if periodic else r[(r >= 0) & (r < nc)]
        cells[i, r] = True
    return cells


def disjoint_batches(x, rk, nc, periodic):
    """Greedy split into batches whose particles' cell boxes do not overlap."""
    ax = [axis_cells(x[:, a], rk, nc, periodic) for a in range(3)]
    batches = []
    for i in range(x.shape[0]):
        for b in batches:
            clash = np.ones(len(b), bool)
            for a in range(3):
                clash &= (ax[a][b] & ax[a][i]).any(axis=1)
            if not clash.any():
                b.append(i)
                break
        else:
            batches.append([i])
    return batches


def gpu_mesh(ctx, mode, x, v, dens, rk, igrp, nc, sign):
    p = api.make_particles(x, v, dens=dens, rk=rk, igrp=igrp)
    if mode == "plain":
        m, t = ctx.assign_on_meshes(p, L, [nc], sign)
        return m[0], t[0]
    if mode == "periodic":
        return ctx.assign_on_global_mesh(p, L, nc, sign, coords=(1, 0, 2))
    return ctx.assign_on_density_mesh(p, L, nc, sign), None


def oracle_mesh(oracle, mode, x, v, dens, rk, igrp, nc, sign, float_weights=True):
    """(FP64 sums of the library's float weights, or the FP64 restatement with
    float_weights=False; FP64 totals) in the GPU call's layout (density-only:
    the n channel)."""
    per = mode == "periodic"
    _, m64, t64 = oracle.assign_on_mesh(x, v, dens, rk, igrp, L, nc, sign, periodic=per,
                                        offset=(L, 0.0, 2 * L), float_weights=float_weights)
    if mode == "density":
        return m64[: nc ** 3], t64
    return m64, t64


@pytest.mark.parametrize("mode", ["plain", "periodic", "density"])
@pytest.mark.parametrize("sign", [-1, 1])
@pytest.mark.parametrize("nc", NCS)
def test_deposit_edges(gpu_ctx, oracle, mode, sign, nc):
    x, v, dens, rk, igrp = edge_inputs()
    if mode == "periodic":  # the periodic deposit takes the particles inside [0, L)
        inside = np.all((x >= 0) & (x < L), axis=1)
        x, v, dens, rk, igrp = x[inside], v[inside], dens[inside], rk[inside], igrp[inside]
    nm = nc ** 3

    # one weight per cell, then the whole set: the oracle's FP64 sums of the
    # library's cell weights to DEP_TOL
    batches = disjoint_batches(x, rk, nc, mode == "periodic")
    assert len(batches) < len(x)  # the batches do combine particles
    for b in batches + [np.arange(len(x))]:
        b = np.asarray(b)
        got, tot = gpu_mesh(gpu_ctx, mode, x[b], v[b], dens[b], rk[b], igrp[b], nc, sign)
        s64, t64 = oracle_mesh(oracle, mode, x[b], v[b], dens[b], rk[b], igrp[b], nc, sign)
        chans = [(0, nm)] if mode == "density" else [(0, nm), (nm, 2 * nm), (2 * nm, 3 * nm)]
        for a, e in chans:
            g, s = got[a:e].astype(np.float64), s64[a:e]
            assert np.all(np.abs(g - s) <= DEP_TOL * np.abs(s)), (mode, sign, nc, a, b[:4])
        if mode != "density":
            vs = s64[3 * nm:]
            scale = np.abs(vs) + np.repeat(s64[:nm], 3)
            assert np.all(np.abs(got[3 * nm:].astype(np.float64) - vs) <= DEP_TOL * scale)
            for k in range(2):
                assert abs(tot[k] - t64[k]) <= TOTAL_TOL * abs(t64[k]), (k, tot, t64)

    # accuracy against the FP64 restatement of the weights
    e64, _ = oracle_mesh(oracle, mode, x, v, dens, rk, igrp, nc, sign, float_weights=False)
    errs = field_errors(got, e64, nc, mode == "density")
    assert max(errs.values()) <= FIELD_TOL, errs


@pytest.mark.parametrize("box,nc", [(100.1, 24), (333.3, 37)])
def test_deposit_box_side_not_a_power_of_two(gpu_ctx, oracle, box, nc):
    """The normalised cell-range edges (x -+ h) / L (coarse_mesh.cpp:72-77) on a
    box side that is not a power of two, where the quotient rounds: particles
    on and next to every cell edge, supports ending on edges.  The cells each
    particle reaches, and so every cell's sum, match the oracle (FP64 sums of
    the library's weights to DEP_TOL, FP64 totals to 1e-12)."""
    rng = np.random.default_rng(5)
    n = 600
    dx = np.float32(np.float32(box) / np.float32(nc))
    edges = np.arange(nc + 1, dtype=np.float32) * dx
    x = rng.choice(edges, (n, 3)).astype(np.float32)
    x += rng.choice(np.float32([-1e-4, 0.0, 1e-4]), (n, 3)).astype(np.float32)
    x[:50] = rng.uniform(0, box, (50, 3)).astype(np.float32)
    rk = (dx * rng.choice(np.float32([0.5, 1.0, 1.5, 2.0, 0.999, 3.0]), n)).astype(np.float32)
    v = rng.normal(size=(n, 3)).astype(np.float32)
    dens = rng.uniform(0.5, 2.0, n).astype(np.float32)
    igrp = rng.choice([-1, 0, 2], n).astype(np.int32)
    p = api.make_particles(x, v, dens=dens, rk=rk, igrp=igrp)
    m, t = gpu_ctx.assign_on_meshes(p, float(np.float32(box)), [nc], -1)
    _, s64, t64 = oracle.assign_on_mesh(x, v, dens, rk, igrp, float(np.float32(box)), nc, -1,
                                        float_weights=True)
    got, nm = m[0].astype(np.float64), nc ** 3
    # a cell below float32's normal range (a sliver of a support's edge can
    # weigh 1e-40) is held to DEP_TOL of the smallest normal float, since a
    # subnormal float carries fewer significant bits
    tiny = float(np.finfo(np.float32).tiny)
    for a, e in ((0, nm), (nm, 2 * nm), (2 * nm, 3 * nm)):
        s = s64[a:e]
        assert np.all(np.abs(got[a:e] - s) <= DEP_TOL * np.maximum(np.abs(s), tiny))
    for k in range(2):
        assert abs(t[0][k] - t64[k]) <= TOTAL_TOL * abs(t64[k])
