"""Python mirror of the reference's hot-path interface, backed by the GB300
C ABI (include/asmooth_gb300.h).

Particles are numpy structured arrays with the reference's ``struct Particle``
layout (basic_types.h:10-15): ``x`` float32[3], ``v`` float32[3], ``dens``,
``rk`` float32 and ``igrp`` int32, 36 bytes per record.  The functions keep the
reference's names and argument meaning:

  neighbor_search        KDTree::construct + neighbor_search loop
                         (clumping_tree_main.cpp:390-395, :418-430)
  assign_on_mesh         clear_mesh + assign_on_mesh (coarse_mesh.cpp:24-127)
  assign_on_global_mesh  periodic variant (global_mesh.cpp:25-123)
  assign_on_density_mesh n-only variant (coarse_mesh.cpp:212-269)
  mesh_total             FP64 totals (coarse_mesh.cpp:35-43)
  normalise_mesh         write_mesh_separate normalisation (coarse_mesh.cpp:158-171)
  group_fof, remove_small_groups (fof.cpp:34-166)
  mark_halo_particles    SO-halo loop (clumping_tree_main.cpp:465-485)
  write_mesh_separate, write_mesh (coarse_mesh.cpp:128-208)
  write_fof_halos        FOF catalogue file (fof.cpp:169-219)

Where the reference asserts or aborts, these raise :class:`AsmoothError`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

PARTICLE_DTYPE = np.dtype([("x", "<f4", (3,)), ("v", "<f4", (3,)), ("dens", "<f4"),
                           ("rk", "<f4"), ("igrp", "<i4")])
HALO_DTYPE = np.dtype([("x", "<f4", (3,)), ("r", "<f4"), ("mass", "<f4")])
# struct FofHalo (fof.cpp:22-25), the record of the FOF catalogue file
FOF_HALO_DTYPE = np.dtype([("x", "<f4", (3,)), ("v", "<f4", (3,)), ("nfof", "<i4")])
assert FOF_HALO_DTYPE.itemsize == 28
assert PARTICLE_DTYPE.itemsize == 36 and HALO_DTYPE.itemsize == 20

ASG_OK = 0
ASG_ERR_ARG, ASG_ERR_CUDA, ASG_ERR_NOMEM, ASG_ERR_FEW, ASG_ERR_ZERO_RK = -1, -2, -3, -4, -5
ASG_ERR_NONFINITE, ASG_ERR_STACK, ASG_ERR_TIES, ASG_ERR_RANGE, ASG_ERR_STATE = -6, -7, -8, -9, -10
ASG_ERR_UNIONFIND = -11
ASG_ERR_NOALLOC_LIMIT = -12
ASG_ERR_IO = -13


class AsmoothError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


def make_particles(x, v=None, dens=None, rk=None, igrp=None) -> np.ndarray:
    """Build a Particle record array (the reader's state: dens = rk = igrp = 0)."""
    x = np.asarray(x, np.float32)
    p = np.zeros(x.shape[0], PARTICLE_DTYPE)
    p["x"] = x
    if v is not None:
        p["v"] = v
    if dens is not None:
        p["dens"] = dens
    if rk is not None:
        p["rk"] = rk
    if igrp is not None:
        p["igrp"] = igrp
    return p


class _HostBlock:
    """A block from asg_host_alloc, freed when the last array over it goes."""

    def __init__(self, nbytes: int):
        self._lib = _lib.load()
        p = C.c_void_p()
        rc = self._lib.asg_host_alloc(int(nbytes), C.byref(p))
        if rc != 0 or not p.value:
            raise MemoryError(f"asg_host_alloc({nbytes}): host memory could not be mapped "
                              f"or pinned (status {rc}; pinning needs the CUDA driver)")
        self.ptr = p.value
        self.__array_interface__ = {"shape": (int(nbytes),), "typestr": "|u1",
                                    "data": (self.ptr, False), "version": 3}

    def __del__(self):
        if getattr(self, "ptr", None):
            self._lib.asg_host_free(C.c_void_p(self.ptr))
            self.ptr = None


def host_array(shape, dtype=np.float32) -> np.ndarray:
    """A zeroed C-contiguous array in huge-page pinned host memory
    (asg_host_alloc): host<->device copies from and to it keep the link's
    rate on multi-GB transfers.  Use it for the particle records and meshes
    passed to ``Context.smooth`` and the other host-array calls."""
    dtype = np.dtype(dtype)
    shape = (shape,) if np.isscalar(shape) else tuple(shape)
    n = int(np.prod(shape, dtype=np.int64)) * dtype.itemsize
    return np.asarray(_HostBlock(max(n, 1)))[:n].view(dtype).reshape(shape)


def make_halos(x, r, mass) -> np.ndarray:
    h = np.zeros(len(r), HALO_DTYPE)
    h["x"] = np.asarray(x, np.float32).reshape(-1, 3)
    h["r"] = r
    h["mass"] = mass
    return h


def _ptr(a) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


def _check_particles(p: np.ndarray) -> np.ndarray:
    if not isinstance(p, np.ndarray) or p.dtype != PARTICLE_DTYPE or not p.flags.c_contiguous:
        raise TypeError("particles must be a C-contiguous array of PARTICLE_DTYPE")
    return p


class Context:
    """One library context: a CUDA stream and device buffers on one GPU."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.asg_create(C.byref(h), int(device))
        if rc != ASG_OK:
            raise AsmoothError(rc, self.lib.asg_strerror(rc).decode())
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.lib.asg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ok(self, rc: int):
        if rc != ASG_OK:
            msg = self.lib.asg_strerror(rc).decode()
            detail = self.lib.asg_last_error(self.h).decode()
            raise AsmoothError(rc, f"{msg}: {detail}")

    @property
    def kernel_launches(self) -> int:
        return int(self.lib.asg_kernel_launches(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.asg_stream(self.h) or 0)

    def set_timing(self, enable: bool = True):
        self._ok(self.lib.asg_set_timing(self.h, int(bool(enable))))

    def phase_ms(self) -> dict:
        ms = np.zeros(_lib.NPHASES, np.float64)
        self._ok(self.lib.asg_phase_ms(self.h, _ptr(ms)))
        return {self.lib.asg_phase_name(i).decode(): float(ms[i]) for i in range(_lib.NPHASES)}

    def deposit_stats(self) -> dict:
        c, b, i = C.c_longlong(0), C.c_longlong(0), C.c_longlong(0)
        self._ok(self.lib.asg_deposit_stats(self.h, C.byref(c), C.byref(b), C.byref(i)))
        return {"candidates": c.value, "buckets": b.value, "items": i.value}

    def measure_fp32_peak(self) -> float:
        t = C.c_double(0.0)
        self._ok(self.lib.asg_measure_fp32_peak(self.h, C.byref(t)))
        return t.value

    # ---- reference-shaped calls (host arrays, in place) -------------------------
    def neighbor_search(self, p: np.ndarray, left: float, right: float) -> np.ndarray:
        _check_particles(p)
        self._ok(self.lib.asg_neighbor_search(self.h, _ptr(p), len(p), left, right))
        return p

    def assign_on_meshes(self, p: np.ndarray, boxsize: float, ncs, sign: int = 1,
                         periodic: bool = False, coords=(0, 0, 0)):
        _check_particles(p)
        ncs = [int(nc) for nc in ncs]
        meshes = [np.zeros(6 * nc ** 3, np.float32) for nc in ncs]
        arr = (C.c_void_p * len(ncs))(*[m.ctypes.data for m in meshes])
        nca = np.asarray(ncs, np.int32)
        co = np.asarray(coords, np.int32)
        tot = np.zeros(2 * len(ncs), np.float64)
        self._ok(self.lib.asg_assign_on_meshes(self.h, _ptr(p), len(p), boxsize, _ptr(nca), len(ncs),
                                               int(sign), int(bool(periodic)), _ptr(co), arr,
                                               _ptr(tot)))
        return meshes, tot.reshape(-1, 2)

    def assign_on_mesh(self, p: np.ndarray, boxsize: float, nc: int, sign: int = 1):
        meshes, tot = self.assign_on_meshes(p, boxsize, [nc], sign)
        return meshes[0], tot[0]

    def assign_on_global_mesh(self, p: np.ndarray, boxsize: float, nc: int, sign: int = 1,
                              coords=(0, 0, 0)):
        meshes, tot = self.assign_on_meshes(p, boxsize, [nc], sign, periodic=True, coords=coords)
        return meshes[0], tot[0]

    def assign_on_density_mesh(self, p: np.ndarray, boxsize: float, nc: int, sign: int = 1):
        _check_particles(p)
        mesh = np.zeros(nc ** 3, np.float32)
        self._ok(self.lib.asg_assign_on_density_mesh(self.h, _ptr(p), len(p), boxsize, int(nc),
                                                     int(sign), _ptr(mesh)))
        return mesh

    def normalise_mesh(self, mesh: np.ndarray, nc: int, boxsize: float) -> np.ndarray:
        m = np.ascontiguousarray(mesh, np.float32).copy()
        self._ok(self.lib.asg_normalise_mesh(self.h, _ptr(m), int(nc), boxsize))
        return m

    def group_fof(self, p: np.ndarray, left: float, right: float, ll: float) -> int:
        _check_particles(p)
        ng = C.c_int(0)
        self._ok(self.lib.asg_group_fof(self.h, _ptr(p), len(p), left, right, ll, C.byref(ng)))
        return ng.value

    def remove_small_groups(self, p: np.ndarray, ngrp: int) -> int:
        _check_particles(p)
        nh = C.c_int(0)
        self._ok(self.lib.asg_remove_small_groups(self.h, _ptr(p), len(p), int(ngrp), C.byref(nh)))
        return nh.value

    def mark_halo_particles(self, p: np.ndarray, halos: np.ndarray, left: float, right: float):
        _check_particles(p)
        halos = np.ascontiguousarray(halos, HALO_DTYPE)
        nph = C.c_long(0)
        mh = C.c_double(0.0)
        self._ok(self.lib.asg_mark_halo_particles(self.h, _ptr(p), len(p), _ptr(halos), len(halos),
                                                  left, right, C.byref(nph), C.byref(mh)))
        return nph.value, mh.value

    def smooth(self, p: np.ndarray, left: float, right: float, boxsize: float, ncs,
               sign: int = -1, halos: np.ndarray | None = None, meshes=None):
        """Neighbour search, SO-halo marking and the deposit for every nc in one call."""
        _check_particles(p)
        ncs = [int(nc) for nc in ncs]
        if meshes is None:
            meshes = [np.zeros(6 * nc ** 3, np.float32) for nc in ncs]
        arr = (C.c_void_p * len(ncs))(*[m.ctypes.data for m in meshes])
        nca = np.asarray(ncs, np.int32)
        tot = np.zeros(2 * len(ncs), np.float64)
        nh = 0 if halos is None else len(halos)
        hal = None if halos is None else np.ascontiguousarray(halos, HALO_DTYPE)
        nph = C.c_long(0)
        mh = C.c_double(0.0)
        self._ok(self.lib.asg_smooth(self.h, _ptr(p), len(p), left, right, boxsize, _ptr(hal), nh,
                                     _ptr(nca), len(ncs), int(sign), arr, _ptr(tot), C.byref(nph),
                                     C.byref(mh)))
        return meshes, tot.reshape(-1, 2), nph.value, mh.value

    def smooth_quantised(self, cell: np.ndarray, off: np.ndarray, v: np.ndarray | None,
                         left: float, right: float, cell_size: float, grid: int, boxsize: float,
                         ncs, sign: int = -1, meshes=None, rk=None, dens=None):
        """Mixed-precision form of ``smooth`` (no halo marking): positions as an
        int32 cell index and uint16 offsets (see ``quantised.quantise``).
        Returns (rk, dens, meshes, totals) with rk and dens in input order."""
        cell = np.ascontiguousarray(cell, np.int32)
        off = np.ascontiguousarray(off, np.uint16)
        n = len(cell)
        if off.shape != (n, 3):
            raise ValueError("off must have shape (n, 3)")
        if v is not None:
            v = np.ascontiguousarray(v, np.float32)
        ncs = [int(nc) for nc in ncs]
        if meshes is None:
            meshes = [np.zeros(6 * nc ** 3, np.float32) for nc in ncs]
        rk = np.zeros(n, np.float32) if rk is None else rk
        dens = np.zeros(n, np.float32) if dens is None else dens
        arr = (C.c_void_p * len(ncs))(*[m.ctypes.data for m in meshes])
        nca = np.asarray(ncs, np.int32)
        tot = np.zeros(2 * len(ncs), np.float64)
        self._ok(self.lib.asg_smooth_quantised(self.h, _ptr(cell), _ptr(off), _ptr(v), n, left,
                                               right, cell_size, int(grid), boxsize, _ptr(nca),
                                               len(ncs), int(sign), _ptr(rk), _ptr(dens), arr,
                                               _ptr(tot)))
        return rk, dens, meshes, tot.reshape(-1, 2)

    # ---- outputs ----------------------------------------------------------------
    def write_mesh_separate(self, base: str, inode: int, mesh: np.ndarray, nc: int,
                            boxsize: float) -> np.ndarray:
        """write_mesh_separate: normalise ``mesh`` in place, write the four files."""
        if mesh.dtype != np.float32 or not mesh.flags.c_contiguous or mesh.size != 6 * nc ** 3:
            raise TypeError("mesh must be a contiguous float32 array of 6*nc^3 values")
        self._ok(self.lib.asg_write_mesh_separate(self.h, base.encode(), int(inode), _ptr(mesh),
                                                  int(nc), boxsize))
        return mesh

    def write_mesh_device(self, k: int, base: str, inode: int):
        self._ok(self.lib.asg_write_mesh_device(self.h, int(k), base.encode(), int(inode)))

    def fof_halos(self, p: np.ndarray, nhalo: int, boxsize: float) -> np.ndarray:
        """write_fof_halos' catalogue (records of FOF_HALO_DTYPE) of labels 1..nhalo."""
        _check_particles(p)
        out = np.zeros(max(int(nhalo), 1), FOF_HALO_DTYPE)
        nl = C.c_int(0)
        self._ok(self.lib.asg_fof_halos(self.h, _ptr(p), len(p), int(nhalo), boxsize, _ptr(out),
                                        C.byref(nl)))
        return out[:nl.value].copy()

    def write_fof_halos(self, filename: str, p: np.ndarray, nhalo: int, boxsize: float):
        _check_particles(p)
        self._ok(self.lib.asg_write_fof_halos(self.h, filename.encode(), _ptr(p), len(p),
                                              int(nhalo), boxsize))

    def run_fof_halos(self, nhalo: int, boxsize: float) -> np.ndarray:
        out = np.zeros(max(int(nhalo), 1), FOF_HALO_DTYPE)
        nl = C.c_int(0)
        self._ok(self.lib.asg_run_fof_halos(self.h, int(nhalo), boxsize, _ptr(out), C.byref(nl)))
        return out[:nl.value].copy()

    # ---- staged device-resident interface ------------------------------------------
    def load_particles(self, p: np.ndarray, left: float, right: float):
        _check_particles(p)
        self._ok(self.lib.asg_load_particles(self.h, _ptr(p), len(p), left, right))

    def load_particles_device(self, x_ptr: int, n: int, left: float, right: float, v_ptr: int = 0,
                              dens_ptr: int = 0, igrp_ptr: int = 0):
        self._ok(self.lib.asg_load_particles_device(self.h, C.c_void_p(x_ptr), C.c_void_p(v_ptr),
                                                    C.c_void_p(dens_ptr), C.c_void_p(igrp_ptr),
                                                    int(n), left, right))

    def load_periodic_cube(self, p: np.ndarray, boxsize: float, buffer_factor: float):
        """The whole box plus its periodic buffer shell built on the device
        (one-rank exchange_buffer + remove_extra_particles); returns
        (np_with_buffers, np_local_kept).  store_particles reads the set back."""
        _check_particles(p)
        nw, nl = C.c_int(0), C.c_int(0)
        self._ok(self.lib.asg_load_periodic_cube(self.h, _ptr(p), len(p), boxsize, buffer_factor,
                                                 C.byref(nw), C.byref(nl)))
        return nw.value, nl.value

    def load_periodic_cube_device(self, x_ptr: int, n: int, boxsize: float, buffer_factor: float,
                                  v_ptr: int = 0):
        nw, nl = C.c_int(0), C.c_int(0)
        self._ok(self.lib.asg_load_periodic_cube_device(self.h, C.c_void_p(x_ptr), C.c_void_p(v_ptr),
                                                        int(n), boxsize, buffer_factor,
                                                        C.byref(nw), C.byref(nl)))
        return nw.value, nl.value

    # ---- particle files decoded on the device ---------------------------------------
    def decode_xv(self, xv: np.ndarray, shift=(0.0, 0.0, 0.0)) -> int:
        """xv payload (n, 6) float32 -> decoded particles kept on the device."""
        xv = np.ascontiguousarray(xv, np.float32).reshape(-1, 6)
        sh = np.asarray(shift, np.float32)
        self._ok(self.lib.asg_decode_xv(self.h, _ptr(xv), len(xv), _ptr(sh)))
        return len(xv)

    def decode_zip(self, zip0: np.ndarray, zip1: np.ndarray, zip2: np.ndarray, zip3: np.ndarray,
                   np_local: int, nc_node_dim: int, mesh_scale: int, v_r2i: float,
                   shift=(0.0, 0.0, 0.0)) -> int:
        z0 = np.ascontiguousarray(zip0, np.uint8)
        z1 = np.ascontiguousarray(zip1, np.int16)
        z2 = np.ascontiguousarray(zip2, np.uint8)
        z3 = np.ascontiguousarray(zip3, np.int32)
        sh = np.asarray(shift, np.float32)
        self._ok(self.lib.asg_decode_zip(self.h, _ptr(z0), _ptr(z1), _ptr(z2), _ptr(z3), z3.size,
                                         int(np_local), int(nc_node_dim), int(mesh_scale),
                                         float(v_r2i), _ptr(sh)))
        return int(np_local)

    def read_pm_file_xv(self, filebase: str, redshift: str, inode: int,
                        shift=(0.0, 0.0, 0.0)) -> int:
        sh = np.asarray(shift, np.float32)
        n = C.c_int(0)
        self._ok(self.lib.asg_read_pm_file_xv(self.h, filebase.encode(), redshift.encode(),
                                              int(inode), _ptr(sh), C.byref(n)))
        return n.value

    def read_pm_file_zip(self, filebase: str, redshift: str, inode: int, nc_node_dim: int,
                         mesh_scale: int, shift=(0.0, 0.0, 0.0)):
        """Returns (np_local, boxsize); the particles stay on the device."""
        sh = np.asarray(shift, np.float32)
        n, L = C.c_int(0), C.c_float(0.0)
        self._ok(self.lib.asg_read_pm_file_zip(self.h, filebase.encode(), redshift.encode(),
                                               int(inode), int(nc_node_dim), int(mesh_scale),
                                               _ptr(sh), C.byref(n), C.byref(L)))
        return n.value, L.value

    def copy_decoded(self, n: int) -> np.ndarray:
        out = np.zeros(int(n), PARTICLE_DTYPE)
        self._ok(self.lib.asg_copy_decoded(self.h, _ptr(out)))
        return out

    def load_decoded_periodic(self, boxsize: float, buffer_factor: float):
        nw, nl = C.c_int(0), C.c_int(0)
        self._ok(self.lib.asg_load_decoded_periodic(self.h, boxsize, buffer_factor, C.byref(nw),
                                                    C.byref(nl)))
        return nw.value, nl.value

    def load_particles_quantised(self, cell: np.ndarray, off: np.ndarray, v: np.ndarray | None,
                                 left: float, right: float, cell_size: float, grid: int):
        cell = np.ascontiguousarray(cell, np.int32)
        off = np.ascontiguousarray(off, np.uint16)
        if off.shape != (len(cell), 3):
            raise ValueError("off must have shape (n, 3)")
        if v is not None:
            v = np.ascontiguousarray(v, np.float32)
        self._ok(self.lib.asg_load_particles_quantised(self.h, _ptr(cell), _ptr(off), _ptr(v),
                                                       len(cell), left, right, cell_size, int(grid)))

    def load_particles_quantised_device(self, cell_ptr: int, off_ptr: int, n: int, left: float,
                                        right: float, cell_size: float, grid: int, v_ptr: int = 0):
        self._ok(self.lib.asg_load_particles_quantised_device(
            self.h, C.c_void_p(cell_ptr), C.c_void_p(off_ptr), C.c_void_p(v_ptr), int(n), left,
            right, cell_size, int(grid)))

    def run_neighbor_search(self):
        self._ok(self.lib.asg_run_neighbor_search(self.h))

    def run_mark_halos(self, halos: np.ndarray):
        halos = np.ascontiguousarray(halos, HALO_DTYPE)
        nph = C.c_long(0)
        mh = C.c_double(0.0)
        self._ok(self.lib.asg_run_mark_halos(self.h, _ptr(halos), len(halos), C.byref(nph),
                                             C.byref(mh)))
        return nph.value, mh.value

    def run_fof(self, ll: float) -> int:
        ng = C.c_int(0)
        self._ok(self.lib.asg_run_fof(self.h, ll, C.byref(ng)))
        return ng.value

    def run_remove_small_groups(self, ngrp: int) -> int:
        nh = C.c_int(0)
        self._ok(self.lib.asg_run_remove_small_groups(self.h, int(ngrp), C.byref(nh)))
        return nh.value

    def run_deposit(self, boxsize: float, ncs, sign: int = -1, periodic: bool = False,
                    coords=(0, 0, 0), density_only: bool = False, want_totals: bool = True):
        ncs = [int(nc) for nc in ncs]
        nca = np.asarray(ncs, np.int32)
        co = np.asarray(coords, np.int32)
        tot = np.zeros(2 * len(ncs), np.float64) if want_totals else None
        self._ok(self.lib.asg_run_deposit(self.h, boxsize, _ptr(nca), len(ncs), int(sign),
                                          int(bool(periodic)), _ptr(co), int(bool(density_only)),
                                          _ptr(tot)))
        return None if tot is None else tot.reshape(-1, 2)

    def run_normalise(self, k: int):
        self._ok(self.lib.asg_run_normalise(self.h, int(k)))

    def mesh_device_ptr(self, k: int) -> int:
        return int(self.lib.asg_mesh_device(self.h, int(k)) or 0)

    def copy_mesh(self, k: int, words: int) -> np.ndarray:
        m = np.zeros(words, np.float32)
        self._ok(self.lib.asg_copy_mesh(self.h, int(k), _ptr(m)))
        return m

    def store_particles(self, p: np.ndarray) -> np.ndarray:
        _check_particles(p)
        self._ok(self.lib.asg_store_particles(self.h, _ptr(p)))
        return p

    def store_fields_device(self, rk_ptr: int = 0, dens_ptr: int = 0, igrp_ptr: int = 0):
        self._ok(self.lib.asg_store_fields_device(self.h, C.c_void_p(rk_ptr), C.c_void_p(dens_ptr),
                                                  C.c_void_p(igrp_ptr)))

    def get_knn(self, n: int):
        t33 = np.zeros(n, np.float32)
        idx33 = np.zeros(n, np.int32)
        self._ok(self.lib.asg_get_knn(self.h, _ptr(t33), _ptr(idx33)))
        return t33, idx33


class Batch:
    """The batched form: many cubes (``synthetic.Cube``-like objects with x, v,
    n, n_local, left, right, boxsize) through the whole path in one CUDA graph,
    on one context (used exclusively until ``close``)."""

    def __init__(self, ctx: Context, cubes, ncs, sign: int = -1):
        self.ctx, self.lib = ctx, ctx.lib
        self.ncs = [int(nc) for nc in ncs]
        self.n = [int(c.n) for c in cubes]
        arr = lambda vals, dt: np.asarray(vals, dt)  # noqa: E731
        npa, nla = arr(self.n, np.int32), arr([c.n_local for c in cubes], np.int32)
        lf, rt = arr([c.left for c in cubes], np.float32), arr([c.right for c in cubes], np.float32)
        bx, nca = arr([c.boxsize for c in cubes], np.float32), arr(self.ncs, np.int32)
        h = C.c_void_p()
        ctx._ok(self.lib.asg_batch_create(ctx.h, len(cubes), _ptr(npa), _ptr(nla), _ptr(lf), _ptr(rt),
                                          _ptr(bx), _ptr(nca), len(self.ncs), int(sign), C.byref(h)))
        self.h = h
        for i, c in enumerate(cubes):
            self.set_item(i, c.x, c.v)

    def set_item(self, i: int, x: np.ndarray, v: np.ndarray | None = None):
        x = np.ascontiguousarray(x, np.float32)
        v = None if v is None else np.ascontiguousarray(v, np.float32)
        if x.shape != (self.n[i], 3):
            raise ValueError("item size is fixed at creation")
        self.ctx._ok(self.lib.asg_batch_set_item(self.h, int(i), _ptr(x), _ptr(v), 0))

    def set_item_quantised(self, i: int, cell: np.ndarray, off: np.ndarray,
                           v: np.ndarray | None, cell_size: float, grid: int):
        """Item i in the mixed-precision form (asg_batch_set_item_quantised)."""
        cell = np.ascontiguousarray(cell, np.int32)
        off = np.ascontiguousarray(off, np.uint16)
        v = None if v is None else np.ascontiguousarray(v, np.float32)
        if cell.shape != (self.n[i],) or off.shape != (self.n[i], 3):
            raise ValueError("item size is fixed at creation")
        self.ctx._ok(self.lib.asg_batch_set_item_quantised(self.h, int(i), _ptr(cell), _ptr(off),
                                                           _ptr(v), float(cell_size), int(grid), 0))

    def set_streams(self, streams: int):
        self.ctx._ok(self.lib.asg_batch_set_streams(self.h, int(streams)))

    def tune(self):
        leaf, seg = C.c_int(0), C.c_int(0)
        self.ctx._ok(self.lib.asg_batch_tune(self.h, C.byref(leaf), C.byref(seg)))
        return leaf.value, seg.value

    def config(self) -> dict:
        """The configuration the batch runs with (tuned or default)."""
        v = [C.c_int(0) for _ in range(4)]
        self.ctx._ok(self.lib.asg_batch_config(self.h, *[C.byref(x) for x in v]))
        return {"leaf": v[0].value, "seg": v[1].value, "knn_warps": v[2].value,
                "deposit_engine": {0: "cuda cores", 1: "tensor cores, 1 warp per item",
                                   2: "tensor cores, 2 warps per item"}.get(v[3].value, v[3].value)}

    def run(self):
        self.ctx._ok(self.lib.asg_batch_run(self.h))

    def stats(self) -> dict:
        ms, k, nl = C.c_double(0.0), C.c_longlong(0), C.c_longlong(0)
        self.ctx._ok(self.lib.asg_batch_stats(self.h, C.byref(ms), C.byref(k), C.byref(nl)))
        return {"graph_ms": ms.value, "kernels": k.value, "particles_local": nl.value}

    def get(self, i: int):
        n = self.n[i]
        rk, dens = np.zeros(n, np.float32), np.zeros(n, np.float32)
        meshes = [np.zeros(6 * nc ** 3, np.float32) for nc in self.ncs]
        arrp = (C.c_void_p * len(meshes))(*[m.ctypes.data for m in meshes])
        tot = np.zeros(2 * len(self.ncs), np.float64)
        self.ctx._ok(self.lib.asg_batch_get(self.h, int(i), _ptr(rk), _ptr(dens), arrp, _ptr(tot)))
        return rk, dens, meshes, tot.reshape(-1, 2)

    def close(self):
        if getattr(self, "h", None):
            self.lib.asg_batch_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


_DEFAULT: Context | None = None


def default_context() -> Context:
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Context(0)
    return _DEFAULT


# module-level names of the reference functions
def neighbor_search(p, left, right):
    return default_context().neighbor_search(p, left, right)


def assign_on_mesh(p, boxsize, nc, sign=1):
    return default_context().assign_on_mesh(p, boxsize, nc, sign)


def assign_on_global_mesh(p, boxsize, nc, sign=1, coords=(0, 0, 0)):
    return default_context().assign_on_global_mesh(p, boxsize, nc, sign, coords)


def assign_on_density_mesh(p, boxsize, nc, sign=1):
    return default_context().assign_on_density_mesh(p, boxsize, nc, sign)


def mesh_total(mesh, nc) -> float:
    """FP64 sum of the first nc^3 floats, as mesh_total (coarse_mesh.cpp:35-43)."""
    return float(np.sum(np.asarray(mesh[: nc ** 3], np.float64)))


def normalise_mesh(mesh, nc, boxsize):
    return default_context().normalise_mesh(mesh, nc, boxsize)


def group_fof(p, left, right, ll):
    return default_context().group_fof(p, left, right, ll)


def remove_small_groups(p, ngrp):
    return default_context().remove_small_groups(p, ngrp)


def mark_halo_particles(p, halos, left, right):
    return default_context().mark_halo_particles(p, halos, left, right)


def write_mesh_separate(base, inode, mesh, nc, boxsize):
    return default_context().write_mesh_separate(base, inode, mesh, nc, boxsize)


def write_mesh(filename, mesh, nc, boxsize):
    """write_mesh (coarse_mesh.cpp:128-143); host only, needs no GPU."""
    m = np.ascontiguousarray(mesh, np.float32)
    if m.size != 6 * nc ** 3:
        raise ValueError("mesh must hold 6*nc^3 floats")
    rc = _lib.load().asg_write_mesh(filename.encode(), _ptr(m), int(nc), float(boxsize))
    if rc:
        raise AsmoothError(rc, f"write_mesh {filename}")


def write_fof_halos(filename, p, nhalo, boxsize):
    return default_context().write_fof_halos(filename, p, nhalo, boxsize)
