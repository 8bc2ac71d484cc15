"""Shared checks for the parity tests."""
import numpy as np


def d2_to_all(x: np.ndarray, q: np.ndarray) -> np.ndarray:
    """Squared distances from point q to every row of x with the reference's
    float32 expression order ((dx*dx + dy*dy) + dz*dz), numpy float32 (no FMA)."""
    x = x.astype(np.float32, copy=False)
    dx = (np.float32(q[0]) - x[:, 0]).astype(np.float32)
    dy = (np.float32(q[1]) - x[:, 1]).astype(np.float32)
    dz = (np.float32(q[2]) - x[:, 2]).astype(np.float32)
    return ((dx * dx + dy * dy) + dz * dz).astype(np.float32)


def set_from_key(x: np.ndarray, q: int, t33: float, idx33: int) -> np.ndarray:
    """The 33 members of query q defined by its 33rd key (t33, idx33)."""
    d2 = d2_to_all(x, x[q])
    idx = np.arange(x.shape[0])
    m = (d2 < np.float32(t33)) | ((d2 == np.float32(t33)) & (idx <= idx33))
    return np.sort(idx[m])


def exact_t33(x: np.ndarray, q: int):
    """Brute-force 33rd key (d2, index) of query q."""
    d2 = d2_to_all(x, x[q])
    order = np.lexsort((np.arange(x.shape[0]), d2))
    k = order[32]
    return d2[k], int(k)


def rel_err_cells(got: np.ndarray, ref: np.ndarray, weight: np.ndarray, frac: float = 1e-3):
    """Max relative error over cells whose weight exceeds frac x mean weight."""
    sel = weight > frac * weight.mean()
    if not sel.any():
        return 0.0
    return float(np.max(np.abs(got[sel].astype(np.float64) - ref[sel]) / np.abs(ref[sel])))


# The deposit's per-cell error against the FP64 sums of its own cell weights
# (products of its float 1-D weights): 3xTF32 tensor-core products (at most
# 2^-21 relative) plus at most 24 FP32 accumulator roundings (2^-23 each)
# between two flushes into double-float sums.
DEP_TOL = 4e-6

# adversarial deposit inputs: a box of side EDGE_L meshed at EDGE_NCS (cells of 4
# and 2 units, 8-cell tiles of 32 and 16 units)
EDGE_L = 64.0
EDGE_NCS = (16, 32)


def edge_inputs(seed=11, n=400):
    """Particles on and next to every cell edge of nc = 32, some past the faces,
    with supports that end on edges; v, dens and halo labels (both signs)."""
    rng = np.random.default_rng(seed)
    edges = np.arange(0, 33, dtype=np.float32) * np.float32(2.0)  # every cell edge of nc = 32
    x = rng.choice(edges, (n, 3)).astype(np.float32)
    x[:100] += rng.choice([-1e-3, 0.0, 1e-3], (100, 3)).astype(np.float32)  # next to edges
    x[100:120] = rng.uniform(-3, EDGE_L + 3, (20, 3)).astype(np.float32)  # past the faces
    rk = rng.choice(np.float32([2.0, 4.0, 6.0, 8.0, 3.999, 0.5, 1.0]), n).astype(np.float32)
    v = rng.normal(size=(n, 3)).astype(np.float32)
    dens = rng.uniform(0.5, 2.0, n).astype(np.float32)
    igrp = rng.choice([-1, 0, 2], n).astype(np.int32)
    return x, v, dens, rk, igrp


def field_errors(got, m64, nc, density_only):
    """Largest relative errors per channel against FP64 on the cells above
    1e-3 of the mean density (v against |v| + n)."""
    nm = nc ** 3
    n64 = m64[:nm]
    if density_only:
        cut = 1e-3 * n64.mean()
        sel = n64 > cut
        return {"n": float(np.max(np.abs(got[sel] - n64[sel]) / n64[sel]))}
    h64, c64, v64 = m64[nm:2 * nm], m64[2 * nm:3 * nm], m64[3 * nm:]
    cut = 1e-3 * float((n64 + h64).mean())
    out = {}
    for name, a, e, ref, dens in (("n", 0, nm, n64, n64), ("halo", nm, 2 * nm, h64, h64),
                                  ("c", 2 * nm, 3 * nm, c64, n64)):
        sel = dens > cut
        g = got[a:e].astype(np.float64)
        out[name] = float(np.max(np.abs(g[sel] - ref[sel]) / np.abs(ref[sel]))) if sel.any() else 0.0
    sel = np.repeat(n64 > cut, 3)  # v against |v| + n on the same cells
    scale = (np.abs(v64) + np.repeat(n64, 3))[sel]
    out["v"] = float(np.max(np.abs(got[3 * nm:].astype(np.float64)[sel] - v64[sel]) / scale))
    return out
