"""Generate the golden fixtures from the REFERENCE itself.

Runs the reference's own hot-path functions (compiled from the reference
sources into oracle/_ref by oracle/build_ref.sh; serial, -ffp-contract=off) on
two small seeded node-cubes and stores inputs and outputs as compressed npz.
Usage: python tests/golden/make_golden.py <reference checkout, e.g. /root/reference>


  plummer_s4.npz  Plummer-sphere cube (side 32, 16^3 particles + 8-unit shell)
  nfw_s16.npz     NFW-halo cube       (side 32, 16^3 particles + 8-unit shell)

Each holds: positions/velocities, rk and dens from neighbor_search, the 33
neighbour indices of a sample of queries, SO-halo marking, the meshes from
assign_on_mesh (sign -1) with their mesh_total values, the normalised meshes
(write_mesh_separate), a periodic global mesh, a density-only mesh, FOF labels
(ll = 0.4) and remove_small_groups.  Re-run with
    python tests/golden/make_golden.py
in a checkout where the reference sources are available.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402
from asmooth_gb300 import synthetic as syn  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
LL = np.float32(2.0 * np.float32(0.2))  # clumping_tree_main.cpp:110 with -l 0.2


def make(name: str, cube: syn.Cube, ncs, seed: int) -> None:
    R = po.Reference()
    x, v = cube.x, cube.v
    n = cube.n
    out = dict(x=x, v=v, n_local=cube.n_local, boxsize=np.float32(cube.boxsize),
               left=np.float32(cube.left), right=np.float32(cube.right), ncs=np.asarray(ncs, np.int32))
    rk, dens, nbr, d2 = R.neighbor_search(x, cube.left, cube.right, want_nbr=True)
    out.update(rk=rk, dens=dens)
    rng = np.random.default_rng(seed)
    sample = np.sort(rng.choice(n, size=min(n, 1500), replace=False)).astype(np.int32)
    out.update(nbr_sample=sample, nbr=np.sort(nbr[sample], axis=1).astype(np.int32))
    # SO halos: some centred on particles, radii 0.5..3, Bryan-Norman-like masses
    nh = 24
    cen = x[rng.choice(cube.n_local, nh, replace=False)] + rng.normal(0, 0.3, (nh, 3)).astype(np.float32)
    halos = np.zeros((nh, 5), np.float32)
    halos[:, :3] = cen
    halos[:, 3] = rng.uniform(0.5, 3.0, nh)
    halos[:, 4] = rng.uniform(10.0, 2000.0, nh)
    halos[0, :3] = cube.right + 1.0  # one outside the cube: skipped
    igrp, np_halo, m_halo = R.mark_halo_particles(x, cube.left, cube.right, halos)
    out.update(halos=halos, igrp_marked=igrp, np_halo=np.int64(np_halo), m_halo=np.float64(m_halo))
    tmp = tempfile.mkdtemp()
    for nc in ncs:
        mesh = R.assign_on_mesh(x, v, dens, rk, igrp, cube.boxsize, nc, -1)
        out[f"mesh{nc}"] = mesh
        out[f"total{nc}"] = np.array([R.mesh_total(mesh, nc), R.mesh_total(mesh[nc ** 3:], nc)])
        out[f"norm{nc}"] = R.write_mesh_separate(os.path.join(tmp, f"m{nc}_"), 0, mesh, nc,
                                                 cube.boxsize)
    nc0 = int(ncs[0])
    out[f"global{nc0}"] = R.assign_on_global_mesh(x, v, dens, rk, igrp, cube.boxsize, nc0, -1,
                                                   (1, 0, 2))
    out[f"density{nc0}"] = R.assign_on_density_mesh(x, rk, igrp, cube.boxsize, nc0, -1)
    g, ng = R.group_fof(x, cube.left, cube.right, LL)
    h, nhalo = R.remove_small_groups(g, ng)
    out.update(ll=LL, fof=po.canonical_groups(g).astype(np.int32), ngroup=np.int32(ng),
               fof_halo=po.canonical_groups(h).astype(np.int32), nhalo=np.int32(nhalo))
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **out)
    print(f"wrote {path}: n={n} ngroup={ng} nhalo={nhalo} np_halo={np_halo} "
          f"({os.path.getsize(path) / 1e6:.2f} MB)")


def main():
    # the reference checkout: first argument or $ASMOOTH_REFERENCE
    if not po.build_reference(sys.argv[1] if len(sys.argv) > 1 else None):
        sys.exit("reference sources not available: cannot regenerate golden fixtures")
    cube, ncs = syn.make_workload("cfg1", scale=4)
    make("plummer_s4.npz", cube, ncs, 11)
    cube, ncs = syn.make_workload("cfg2", scale=16)
    make("nfw_s16.npz", cube, ncs, 12)


if __name__ == "__main__":
    main()
