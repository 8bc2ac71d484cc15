"""Seeded synthetic cubep3m node-cubes for the smoothing path.

No public dataset is involved: these generators stand in for cubep3m snapshots
with the shapes, sizes and clustering the workloads are quoted on (uniform
background plus Plummer or NFW halos, mean particle separation 2 in internal
units).  Positions and velocities are float32.

The periodic buffer shell reproduces what the reference does with one MPI rank:
``exchange_buffer`` (exchange_buffer.cpp:6-11 bins, :112-151 self-exchange with
coordinate shift ``x -= (dn-1)*boxsize``) followed by ``remove_extra_particles``
(clumping_tree_main.cpp:550-576, strict ``(-b, L+b)`` box).  The copies are
appended after the interior particles; their order inside the shell is by
(source bin, direction, input index), which no output of the path depends on.
"""
from __future__ import annotations

import dataclasses
import struct

import numpy as np

__all__ = [
    "Cube",
    "uniform_cube",
    "plummer_cube",
    "nfw_cube",
    "add_periodic_shell",
    "quantise_positions",
    "write_xv",
    "read_xv",
    "make_workload",
]


@dataclasses.dataclass
class Cube:
    """One node-cube: ``x``/``v`` (n,3) float32, ``n_local`` interior particles
    first, then the shell copies; ``boxsize`` L and shell width ``buffer``."""

    x: np.ndarray
    v: np.ndarray
    n_local: int
    boxsize: float
    buffer: float

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    @property
    def left(self) -> float:
        return float(np.float32(-self.buffer))

    @property
    def right(self) -> float:
        return float(np.float32(self.boxsize) + np.float32(self.buffer))


def _dedup(x: np.ndarray, rng: np.random.Generator, boxsize: float) -> np.ndarray:
    """Re-draw exact duplicate positions (a midpoint tree cannot split them)."""
    for _ in range(100):
        v = np.ascontiguousarray(x).view(np.dtype((np.void, 12))).ravel()
        _, first = np.unique(v, return_index=True)
        if first.size == x.shape[0]:
            return x
        dup = np.ones(x.shape[0], bool)
        dup[first] = False
        x[dup] = rng.uniform(0, boxsize, (int(dup.sum()), 3)).astype(np.float32)
    raise RuntimeError("could not remove duplicate positions")


def _wrap(x: np.ndarray, boxsize: float) -> np.ndarray:
    x = np.mod(x, boxsize)
    x[x >= boxsize] = 0.0  # mod of a tiny negative can round up to L
    return x.astype(np.float32)


def uniform_cube(n: int, boxsize: float, seed: int) -> tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, boxsize, (n, 3)).astype(np.float32)
    x = _dedup(_wrap(x, boxsize), rng, boxsize)
    v = rng.normal(0, 1, (n, 3)).astype(np.float32)
    return x, v


def plummer_cube(n: int, boxsize: float, seed: int, frac_halo: float = 0.5,
                 n_spheres: int = 200, a_range=(0.5, 4.0)) -> tuple[np.ndarray, np.ndarray]:
    """Uniform background + ``n_spheres`` Plummer spheres (centres uniform, scale
    radius log-uniform in ``a_range``, r = a / sqrt(u^(-2/3) - 1)), periodic."""
    rng = np.random.default_rng(seed)
    n_h = int(round(n * frac_halo))
    n_u = n - n_h
    xu = rng.uniform(0, boxsize, (n_u, 3))
    centres = rng.uniform(0, boxsize, (n_spheres, 3))
    scale = np.exp(rng.uniform(np.log(a_range[0]), np.log(a_range[1]), n_spheres))
    owner = rng.integers(0, n_spheres, n_h)
    u = rng.uniform(1e-12, 1.0 - 1e-9, n_h)
    r = scale[owner] / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
    d = rng.normal(size=(n_h, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    xh = centres[owner] + d * r[:, None]
    x = _wrap(np.concatenate([xu, xh]), boxsize)
    x = _dedup(x, rng, boxsize)
    v = rng.normal(0, 1, (n, 3)).astype(np.float32)
    return x, v


def _nfw_m(x):
    return np.log1p(x) - x / (1.0 + x)


def _nfw_inverse(target, c, iters=60):
    """Solve m(x) = target on [0, c] by bisection (vectorised)."""
    lo = np.zeros_like(target)
    hi = c.astype(np.float64).copy()
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        below = _nfw_m(mid) < target
        lo = np.where(below, mid, lo)
        hi = np.where(below, hi, mid)
    return 0.5 * (lo + hi)


def nfw_cube(n: int, boxsize: float, seed: int, frac_halo: float = 0.7,
             n_halos: int = 5000, m_range=(1e2, 1e5), c_range=(4.0, 12.0),
             halo_contraction: float = 1.0, return_halos: bool = False):
    """Uniform background + NFW halos: mass log-uniform over ``m_range`` particles
    (normalised so halo members are ``frac_halo`` of n), concentration uniform in
    ``c_range``, r_vir from 200x the mean number density 1/8, radii by inverse-CDF
    sampling of the truncated NFW profile; positions wrapped periodically.
    ``halo_contraction`` scales every halo's radii about its centre."""
    rng = np.random.default_rng(seed)
    n_h = int(round(n * frac_halo))
    n_u = n - n_h
    mass = np.exp(rng.uniform(np.log(m_range[0]), np.log(m_range[1]), n_halos))
    counts = np.floor(mass / mass.sum() * n_h).astype(np.int64)
    short = n_h - int(counts.sum())
    if short > 0:
        counts[np.argsort(-mass)[:short]] += 1
    conc = rng.uniform(c_range[0], c_range[1], n_halos)
    mean_density = 1.0 / 8.0
    r_vir = (3.0 * counts / (4.0 * np.pi * 200.0 * mean_density)) ** (1.0 / 3.0)
    centres = rng.uniform(0, boxsize, (n_halos, 3))
    owner = np.repeat(np.arange(n_halos), counts)
    cc = conc[owner]
    u = rng.uniform(0, 1, owner.size)
    xs = _nfw_inverse(u * _nfw_m(cc), cc)
    r = xs * (r_vir[owner] / cc) * halo_contraction
    d = rng.normal(size=(owner.size, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    xh = centres[owner] + d * r[:, None]
    xu = rng.uniform(0, boxsize, (n_u, 3))
    x = _wrap(np.concatenate([xu, xh]), boxsize)
    x = _dedup(x, rng, boxsize)
    v = rng.normal(0, 1, (n, 3)).astype(np.float32)
    if return_halos:
        return x, v, dict(centre=centres, r_vir=r_vir * halo_contraction, count=counts)
    return x, v


def nfw_cube_device(n: int, boxsize: float, seed: int, frac_halo: float = 0.7,
                    n_halos: int = 5000, m_range=(1e2, 1e5), c_range=(4.0, 12.0),
                    device: str = "cuda"):
    """``nfw_cube``'s model drawn with torch's generator on the device: the
    same halo masses, concentrations, radii and directions by the same
    formulas, in seconds for 512^3 particles where the numpy version takes
    minutes.  The particles differ from ``nfw_cube``'s for the same seed.
    Returns float32 (n, 3) device tensors x in [0, boxsize) and v."""
    import math

    import torch

    g = torch.Generator(device=device)
    g.manual_seed(seed)
    f64 = dict(dtype=torch.float64, device=device)

    def uni(shape, lo, hi):
        return torch.empty(shape, **f64).uniform_(lo, hi, generator=g)

    n_h = int(round(n * frac_halo))
    n_u = n - n_h
    mass = torch.exp(uni(n_halos, math.log(m_range[0]), math.log(m_range[1])))
    counts = torch.floor(mass / mass.sum() * n_h).to(torch.int64)
    short = n_h - int(counts.sum())
    if short > 0:
        counts[torch.argsort(-mass)[:short]] += 1
    conc = uni(n_halos, c_range[0], c_range[1])
    r_vir = (3.0 * counts.double() / (4.0 * math.pi * 200.0 / 8.0)) ** (1.0 / 3.0)
    centres = uni((n_halos, 3), 0.0, boxsize)
    owner = torch.repeat_interleave(torch.arange(n_halos, device=device), counts)
    cc = conc[owner]
    target = uni(owner.numel(), 0.0, 1.0) * (torch.log1p(cc) - cc / (1.0 + cc))
    lo, hi = torch.zeros_like(cc), cc.clone()
    for _ in range(60):  # bisection of m(x) = target, as _nfw_inverse
        mid = 0.5 * (lo + hi)
        below = (torch.log1p(mid) - mid / (1.0 + mid)) < target
        lo = torch.where(below, mid, lo)
        hi = torch.where(below, hi, mid)
    r = 0.5 * (lo + hi) * (r_vir[owner] / cc)
    del lo, hi, target, cc
    d = torch.randn((owner.numel(), 3), generator=g, **f64)
    d /= torch.linalg.norm(d, dim=1, keepdim=True)
    x = torch.cat([uni((n_u, 3), 0.0, boxsize), centres[owner] + d * r[:, None]])
    del d, r, owner
    x = torch.remainder(x, boxsize).float()
    x[x >= boxsize] = 0.0
    for _ in range(100):  # re-draw exact duplicates, as _dedup
        _, inv, cnt = torch.unique(x.view(torch.int32), dim=0, return_inverse=True,
                                   return_counts=True)
        dup = cnt[inv] > 1
        if not bool(dup.any()):
            break
        first = torch.full((cnt.numel(),), x.shape[0], dtype=torch.int64, device=device)
        first.scatter_reduce_(0, inv, torch.arange(x.shape[0], device=device), "amin")
        dup[first] = False
        x[dup] = uni((int(dup.sum()), 3), 0.0, boxsize).float()
    v = torch.randn((n, 3), generator=g, dtype=torch.float32, device=device)
    return x.contiguous(), v


def add_periodic_shell(x: np.ndarray, v: np.ndarray, boxsize: float,
                       buffer: float) -> Cube:
    """One-rank ``exchange_buffer`` + ``remove_extra_particles`` (see module doc)."""
    L = np.float32(boxsize)
    bf = np.float32(np.float32(buffer) / L)  # the reference's buffer_factor
    lt = np.float32(bf * L)
    rt = np.float32(np.float32(1.0 - bf) * L)
    bins = ((x >= lt).astype(np.int64) + (x > rt).astype(np.int64))  # (n,3) in {0,1,2}
    bidx = bins[:, 0] + 3 * bins[:, 1] + 9 * bins[:, 2]
    xs, vs = [x], [v]
    for i in range(27):
        if i == 13:
            continue
        sel = np.nonzero(bidx == i)[0]
        if sel.size == 0:
            continue
        bn = (i % 3, (i // 3) % 3, i // 9)
        for j in range(27):
            if j == 13:
                continue
            dn = (j % 3, (j // 3) % 3, j // 9)
            if all(dn[d] == 1 or dn[d] == bn[d] for d in range(3)):
                y = x[sel].copy()
                for d in range(3):
                    y[:, d] = y[:, d] - np.float32((dn[d] - 1) * L)
                xs.append(y)
                vs.append(v[sel])
    xa = np.concatenate(xs).astype(np.float32)
    va = np.concatenate(vs).astype(np.float32)
    dx = np.float32(bf * L)
    lo, hi = np.float32(-dx), np.float32(L + dx)
    keep = np.all((xa > lo) & (xa < hi), axis=1)
    n_local = int(keep[: x.shape[0]].sum())
    return Cube(np.ascontiguousarray(xa[keep]), np.ascontiguousarray(va[keep]),
                n_local, float(boxsize), float(dx))


def quantise_positions(cube: Cube, cell_size: float = 4.0):
    """Mixed-precision form of a cube's positions (4-unit cells, 16-bit
    offsets): returns (cell, off, grid) as ``quantised.quantise``."""
    from .quantised import quantise

    return quantise(cube.x, cube.left, cube.right, cell_size)


def write_xv(path: str, x: np.ndarray, v: np.ndarray) -> None:
    """cubep3m xv file (file_reader2.cpp:10-15, :43-85): 48-byte header (int
    np_local + 11 floats), then n x [x y z vx vy vz] float32."""
    n = x.shape[0]
    with open(path, "wb") as f:
        f.write(struct.pack("<i11f", n, *([0.0] * 11)))
        f.write(np.concatenate([x, v], axis=1).astype("<f4").tobytes())


def zip_paths(filebase: str, redshift: str, inode: int) -> list[str]:
    """<filebase><inode>/<redshift>zip{0,1,2,3}_<inode>.dat (file_reader2.cpp:155-165)."""
    return [f"{filebase}{inode}/{redshift}zip{k}_{inode}.dat" for k in range(4)]


def xv_path(filebase: str, redshift: str, inode: int) -> str:
    """<filebase><inode>/<redshift>xv<inode>.dat (file_reader2.cpp:33)."""
    return f"{filebase}{inode}/{redshift}xv{inode}.dat"


def write_zip(filebase: str, redshift: str, inode: int, x: np.ndarray, v: np.ndarray,
              nc_node_dim: int, mesh_scale: int, v_r2i: float,
              shift=(0.0, 0.0, 0.0)) -> np.ndarray:
    """cubep3m zipped particles as read by read_pm_file_zip (file_reader2.cpp:90-272),
    little endian: zip0 = 64-byte header (int np_local, float ... v_r2i at word
    12) + 3 uint8 offsets per particle, zip1 = 64-byte header + 3 int16
    velocities, zip2 = one uint8 count per fine cell (x fastest, 255 = the
    count is the next int32 of zip3), zip3 = those int32 counts.  Positions are
    quantised to 1/256 of a cell of side mesh_scale, velocities to 1/v_r2i.
    Returns the input index of each stored particle (storage order = cell order)."""
    import os

    x = np.asarray(x, np.float64) + np.asarray(shift, np.float64)
    n = x.shape[0]
    g = nc_node_dim
    rel = x / mesh_scale
    c = np.clip(np.floor(rel).astype(np.int64), 0, g - 1)
    off = np.clip(np.floor((rel - c) * 256.0), 0, 255).astype(np.uint8)
    cell = (c[:, 2] * g + c[:, 1]) * g + c[:, 0]
    order = np.argsort(cell, kind="stable")
    counts = np.bincount(cell, minlength=g ** 3)
    vi = np.clip(np.rint(np.asarray(v, np.float64) * v_r2i), -32768, 32767).astype("<i2")
    paths = zip_paths(filebase, redshift, inode)
    os.makedirs(os.path.dirname(paths[0]) or ".", exist_ok=True)
    head0 = np.zeros(16, "<f4")
    head0.view("<i4")[0] = n
    head0[12] = v_r2i
    with open(paths[0], "wb") as f:
        f.write(head0.tobytes())
        f.write(off[order].tobytes())
    with open(paths[1], "wb") as f:
        f.write(np.zeros(16, "<f4").tobytes())
        f.write(vi[order].tobytes())
    with open(paths[2], "wb") as f:
        f.write(np.minimum(counts, 255).astype(np.uint8).tobytes())
    with open(paths[3], "wb") as f:
        f.write(counts[counts >= 255].astype("<i4").tobytes())
    return order


def read_xv(path: str) -> tuple[np.ndarray, np.ndarray]:
    with open(path, "rb") as f:
        n = struct.unpack("<i", f.read(4))[0]
        f.read(44)
        a = np.frombuffer(f.read(24 * n), dtype="<f4").reshape(n, 6)
    return a[:, :3].copy(), a[:, 3:].copy()


WORKLOADS = {
    # name: (generator, n per dim, boxsize, ncs)
    "cfg1": ("plummer", 64, 128.0, (32, 64)),
    "cfg2": ("nfw", 256, 512.0, (64, 128, 256)),
    "cfg5": ("nfw", 512, 1024.0, (128, 256, 512)),
}


def _batch_cube(n, box, cseed, f, n_halos, contractions):
    """One cube of the batched workload at every contraction (a pool task)."""
    out = []
    for con in contractions:
        x, v = nfw_cube(n, box, cseed, frac_halo=f, n_halos=n_halos, halo_contraction=con)
        out.append(add_periodic_shell(x, v, box, 8.0))
    return out


def make_batch(seed: int = 4, scale: int = 1, n_cubes: int = 27,
               contractions=(1.0, 0.7, 0.5), workers: int = 1) -> tuple[list, tuple]:
    """The batched workload: ``n_cubes`` node-cubes of side 256 (mean
    separation 2, so 128^3 particles on average), each with its own halo
    fraction f ~ U[0.2, 0.8] and a particle count 128^3 * (1 + (f - 0.5)/2)
    that varies with it, NFW halos as in the 256^3 cube (625 per cube), and
    one item per redshift with every halo contracted by the given factor about
    its centre.  Items are ordered cube-major; nc = 32, 64, 128.  workers > 1
    generates the cubes in a process pool (started with spawn, so it is safe
    after CUDA has been initialised); the items do not depend on it."""
    rng = np.random.default_rng(seed)
    box = 256.0 / scale
    npd = 128 // scale
    tasks = []
    for c in range(n_cubes):
        f = float(rng.uniform(0.2, 0.8))
        n = int(round(npd ** 3 * (1.0 + 0.5 * (f - 0.5))))
        tasks.append((n, box, 1000 * seed + c, f, max(8, 625 // scale ** 3), tuple(contractions)))
    if workers > 1 and n_cubes > 1:
        import concurrent.futures as cf
        import multiprocessing as mp

        with cf.ProcessPoolExecutor(min(workers, n_cubes), mp_context=mp.get_context("spawn")) as ex:
            cubes = list(ex.map(_batch_cube, *zip(*tasks)))
    else:
        cubes = [_batch_cube(*t) for t in tasks]
    items = [it for cube in cubes for it in cube]
    ncs = tuple(max(4, nc // scale) for nc in (32, 64, 128))
    return items, ncs


def make_workload(name: str, seed: int | None = None, scale: int = 1) -> tuple[Cube, tuple]:
    """Build a named workload with its 8-unit periodic shell.  ``scale`` > 1
    divides the particle count per dimension and the box side by ``scale`` (same
    mean separation and clustering model) for quick tests."""
    kind, npd, box, ncs = WORKLOADS[name]
    npd //= scale
    box /= scale
    seed = {"cfg1": 1, "cfg2": 2, "cfg5": 5}[name] if seed is None else seed
    n = npd ** 3
    if kind == "plummer":
        x, v = plummer_cube(n, box, seed)
    else:
        n_halos = 5000 if name == "cfg2" else 20000
        n_halos = max(8, n_halos // scale ** 3)
        x, v = nfw_cube(n, box, seed, n_halos=n_halos)
    cube = add_periodic_shell(x, v, box, 8.0)
    ncs = tuple(max(4, nc // scale) for nc in ncs)
    return cube, ncs
