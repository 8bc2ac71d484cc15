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


def dens_brute(x: np.ndarray, rk: np.ndarray, t33: np.ndarray, idx33: np.ndarray, j: int) -> float:
    """dens of receiver j by brute force: the reference's float32 ker(q, j) of
    every query q whose 32-set ((d2, index) below its 33rd key) holds j,
    summed in float64."""
    d2 = d2_to_all(x, x[j])  # d2(q, j) for every q (the squares of exact negations agree)
    member = (d2 < t33) | ((d2 == t33) & (j < idx33))
    q = np.nonzero(member)[0]
    hinv = (np.float32(1.0) / rk[q].astype(np.float32)).astype(np.float32)
    dx = np.abs(x[q].astype(np.float32) - x[j].astype(np.float32)).astype(np.float32)
    w = (hinv * hinv).astype(np.float32) * hinv
    for a in range(3):
        w = (w * (np.float32(1.0) - (dx[:, a] * hinv).astype(np.float32))).astype(np.float32)
    return float(np.sum(w.astype(np.float64)))


def rel_err_cells(got: np.ndarray, ref: np.ndarray, weight: np.ndarray, frac: float = 1e-3):
    """Max relative error over cells whose weight exceeds frac x mean weight."""
    sel = weight > frac * weight.mean()
    if not sel.any():
        return 0.0
    return float(np.max(np.abs(got[sel].astype(np.float64) - ref[sel]) / np.abs(ref[sel])))
