"""ctypes loader for the CPU oracle (liborc) and the reference harness (oracle/_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of bench.py.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_SO = os.path.join(HERE, "liborc.so")
REF_DIR = os.path.join(HERE, "_ref")
K = 33
# struct FofHalo (fof.cpp:22-25): 28 bytes
FOF_HALO_DTYPE = np.dtype([("x", "<f4", (3,)), ("v", "<f4", (3,)), ("nfof", "<i4")])

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_vp = C.c_void_p


def build_oracle(force: bool = False) -> str:
    """Compile asmooth_oracle.c (gcc, -ffp-contract=off, OpenMP) into liborc.so."""
    src = os.path.join(HERE, "asmooth_oracle.c")
    if force or not os.path.exists(ORC_SO) or os.path.getmtime(ORC_SO) < os.path.getmtime(src):
        tmp = ORC_SO + f".{os.getpid()}.tmp"
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
                               "-fPIC", "-shared", "-o", tmp, src, "-lm"])
        os.replace(tmp, ORC_SO)
    return ORC_SO


def build_reference(ref_dir: str | None = None) -> bool:
    """Compile the reference harness from the reference checkout in ref_dir (or
    $ASMOOTH_REFERENCE) when it is present; True when the harness exists."""
    ref_dir = ref_dir or os.environ.get("ASMOOTH_REFERENCE", "")
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), ref_dir])
    return os.path.exists(os.path.join(REF_DIR, "libasmooth_ref.so"))


def _p(a):
    return None if a is None else a.ctypes.data_as(_vp)


class Oracle:
    def __init__(self):
        build_oracle()
        self.lib = C.CDLL(ORC_SO)
        L = self.lib
        for name in ("orc_neighbor_search", "orc_knn_exact", "orc_dens_from_lists",
                     "orc_assign_on_mesh", "orc_assign_on_mesh_fw", "orc_assign_on_density_mesh",
                     "orc_normalise_mesh",
                     "orc_group_fof", "orc_remove_small_groups", "orc_mark_halo_particles",
                     "orc_fof_halos", "orc_decode_zip"):
            getattr(L, name).restype = C.c_int
        L.orc_mesh_total.restype = C.c_double

    # -- kNN -----------------------------------------------------------------
    def neighbor_search(self, x, left, right, nthreads=1, dens=None, want_nbr=False):
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        rk = np.zeros(n, np.float32)
        dens = np.zeros(n, np.float32) if dens is None else np.array(dens, np.float32)
        nbr = np.zeros((n, K), np.int32) if want_nbr else None
        d2 = np.zeros((n, K), np.float32) if want_nbr else None
        rc = self.lib.orc_neighbor_search(_p(x), C.c_int(n), C.c_float(left), C.c_float(right),
                                          C.c_int(nthreads), _p(rk), _p(dens), _p(nbr), _p(d2))
        if rc:
            raise RuntimeError(f"orc_neighbor_search failed: {rc}")
        return (rk, dens, nbr, d2) if want_nbr else (rk, dens)

    def knn_exact(self, x, left, right, nthreads=os.cpu_count()):
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        t33 = np.zeros(n, np.float32)
        idx33 = np.zeros(n, np.int32)
        nbr = np.zeros((n, K), np.int32)
        rc = self.lib.orc_knn_exact(_p(x), C.c_int(n), C.c_float(left), C.c_float(right),
                                    C.c_int(nthreads), _p(t33), _p(idx33), _p(nbr))
        if rc:
            raise RuntimeError(f"orc_knn_exact failed: {rc}")
        return t33, idx33, nbr

    def dens_from_lists(self, x, nbr, t33):
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        rk = np.zeros(n, np.float32)
        d32 = np.zeros(n, np.float32)
        d64 = np.zeros(n, np.float64)
        rc = self.lib.orc_dens_from_lists(_p(x), C.c_int(n), _p(np.ascontiguousarray(nbr, np.int32)),
                                          _p(np.ascontiguousarray(t33, np.float32)),
                                          _p(rk), _p(d32), _p(d64))
        if rc:
            raise RuntimeError(f"orc_dens_from_lists failed: {rc}")
        return rk, d32, d64

    # -- mesh ----------------------------------------------------------------
    def assign_on_mesh(self, x, v, dens, rk, igrp, boxsize, nc, sign=-1, periodic=False,
                       offset=(0.0, 0.0, 0.0), nthreads=1, want64=True, float_weights=False):
        """(float mesh, FP64 mesh, FP64 totals).  The float mesh is the
        reference's; the FP64 mesh is the FP64 restatement, or with
        float_weights the FP64 sums of the library's cell weights (the
        products of its float 1-D cell integrals, times 1, dens, v).  The
        totals are the FP64 sums of the library's cell weights."""
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        mesh = np.zeros(6 * nc ** 3, np.float32)
        m64 = np.zeros(6 * nc ** 3, np.float64) if want64 else None
        tot = np.zeros(2, np.float64) if want64 else None
        off = np.asarray(offset, np.float32)
        fn = self.lib.orc_assign_on_mesh_fw if float_weights else self.lib.orc_assign_on_mesh
        rc = fn(
            _p(x), _p(np.ascontiguousarray(v, np.float32)), _p(np.ascontiguousarray(dens, np.float32)),
            _p(np.ascontiguousarray(rk, np.float32)), _p(np.ascontiguousarray(igrp, np.int32)),
            C.c_int(n), C.c_float(boxsize), C.c_int(nc), C.c_int(sign), C.c_int(int(periodic)),
            _p(off), C.c_int(nthreads), _p(mesh), _p(m64), _p(tot))
        if rc:
            raise RuntimeError(f"orc_assign_on_mesh failed: {rc}")
        return mesh, m64, tot

    def assign_on_density_mesh(self, x, rk, igrp, boxsize, nc, sign=-1):
        mesh = np.zeros(nc ** 3, np.float32)
        rc = self.lib.orc_assign_on_density_mesh(
            _p(np.ascontiguousarray(x, np.float32)), _p(np.ascontiguousarray(rk, np.float32)),
            _p(np.ascontiguousarray(igrp, np.int32)), C.c_int(x.shape[0]), C.c_float(boxsize),
            C.c_int(nc), C.c_int(sign), _p(mesh))
        if rc:
            raise RuntimeError(f"orc_assign_on_density_mesh failed: {rc}")
        return mesh

    def mesh_total(self, mesh, nc):
        return self.lib.orc_mesh_total(_p(np.ascontiguousarray(mesh, np.float32)), C.c_int(nc))

    def normalise_mesh(self, mesh, nc, boxsize):
        m = np.array(mesh, np.float32)
        rc = self.lib.orc_normalise_mesh(_p(m), C.c_int(nc), C.c_float(boxsize))
        if rc:
            raise RuntimeError("orc_normalise_mesh failed")
        return m

    # -- FOF / halos -----------------------------------------------------------
    def group_fof(self, x, left, right, ll, exact=False):
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        igrp = np.zeros(n, np.int32)
        ng = C.c_int(0)
        rc = self.lib.orc_group_fof(_p(x), C.c_int(n), C.c_float(left), C.c_float(right),
                                    C.c_float(ll), C.c_int(int(exact)), _p(igrp), C.byref(ng))
        if rc:
            raise RuntimeError(f"orc_group_fof failed: {rc}")
        return igrp, ng.value

    def remove_small_groups(self, igrp, ngrp):
        g = np.array(igrp, np.int32)
        nh = C.c_int(0)
        rc = self.lib.orc_remove_small_groups(_p(g), C.c_int(g.size), C.c_int(ngrp), C.byref(nh))
        if rc:
            raise RuntimeError("orc_remove_small_groups failed")
        return g, nh.value

    def decode_zip(self, filebase, redshift, inode, nc_node_dim, mesh_scale, shift=(0, 0, 0)):
        """Read the four zip files and decode them as read_pm_file_zip: (x, v, boxsize)."""
        paths = [f"{filebase}{inode}/{redshift}zip{k}_{inode}.dat" for k in range(4)]
        b0, b1 = open(paths[0], "rb").read(), open(paths[1], "rb").read()
        n = int(np.frombuffer(b0[:4], "<i4")[0])
        v_r2i = float(np.frombuffer(b0[48:52], "<f4")[0])
        off = np.frombuffer(b0[64:], np.uint8).copy()
        vel = np.frombuffer(b1[64:], "<i2").copy()
        c8 = np.frombuffer(open(paths[2], "rb").read(), np.uint8).copy()
        c32 = np.frombuffer(open(paths[3], "rb").read(), "<i4").copy()
        sh = np.asarray(shift, np.float32)
        x = np.zeros((n, 3), np.float32)
        v = np.zeros((n, 3), np.float32)
        rc = self.lib.orc_decode_zip(_p(off), _p(vel), _p(c8), _p(c32), C.c_int(c32.size), C.c_int(n),
                                     C.c_int(nc_node_dim), C.c_int(mesh_scale), C.c_float(v_r2i),
                                     _p(sh), _p(x), _p(v))
        if rc:
            raise RuntimeError("orc_decode_zip failed")
        return x, v, np.float32(mesh_scale * nc_node_dim)

    def fof_halos(self, x, v, igrp, nhalo, boxsize):
        """write_fof_halos' catalogue: records of FOF_HALO_DTYPE, centre inside the cube."""
        x = np.ascontiguousarray(x, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        g = np.ascontiguousarray(igrp, np.int32)
        out = np.zeros(max(nhalo, 1), FOF_HALO_DTYPE)
        nl = C.c_int(0)
        rc = self.lib.orc_fof_halos(_p(x), _p(v), _p(g), C.c_int(g.size), C.c_int(nhalo),
                                    C.c_float(boxsize), _p(out), C.byref(nl))
        if rc:
            raise RuntimeError("orc_fof_halos failed")
        return out[:nl.value].copy()

    def mark_halo_particles(self, x, left, right, halos, igrp=None, exact=False):
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        g = np.zeros(n, np.int32) if igrp is None else np.array(igrp, np.int32)
        h = np.ascontiguousarray(halos, np.float32).reshape(-1, 5)
        nph = C.c_long(0)
        mh = C.c_double(0.0)
        rc = self.lib.orc_mark_halo_particles(_p(x), C.c_int(n), C.c_float(left), C.c_float(right),
                                              _p(h), C.c_int(h.shape[0]), C.c_int(int(exact)),
                                              _p(g), C.byref(nph), C.byref(mh))
        if rc:
            raise RuntimeError("orc_mark_halo_particles failed")
        return g, nph.value, mh.value


class Reference:
    """The reference's own functions (oracle/_ref), available where the reference
    checkout was present at build time."""

    def __init__(self, omp: bool = False):
        so = os.path.join(REF_DIR, "libasmooth_ref_omp.so" if omp else "libasmooth_ref.so")
        if not os.path.exists(so):
            raise FileNotFoundError(so)
        self.lib = C.CDLL(so)
        self.lib.ref_mesh_total.restype = C.c_double

    @staticmethod
    def available(omp: bool = False) -> bool:
        return os.path.exists(os.path.join(REF_DIR, "libasmooth_ref_omp.so" if omp else "libasmooth_ref.so"))

    def neighbor_search(self, x, left, right, dens=None, want_nbr=False):
        x = np.ascontiguousarray(x, np.float32)
        n = x.shape[0]
        rk = np.zeros(n, np.float32)
        dens = np.zeros(n, np.float32) if dens is None else np.array(dens, np.float32)
        nbr = np.zeros((n, K), np.int32) if want_nbr else None
        d2 = np.zeros((n, K), np.float32) if want_nbr else None
        self.lib.ref_neighbor_search(_p(x), C.c_int(n), C.c_float(left), C.c_float(right),
                                     _p(rk), _p(dens), _p(nbr), _p(d2))
        return (rk, dens, nbr, d2) if want_nbr else (rk, dens)

    def assign_on_mesh(self, x, v, dens, rk, igrp, boxsize, nc, sign=-1):
        mesh = np.zeros(6 * nc ** 3, np.float32)
        self.lib.ref_assign_on_mesh(
            _p(np.ascontiguousarray(x, np.float32)), _p(np.ascontiguousarray(v, np.float32)),
            _p(np.ascontiguousarray(dens, np.float32)), _p(np.ascontiguousarray(rk, np.float32)),
            _p(np.ascontiguousarray(igrp, np.int32)), C.c_int(x.shape[0]), C.c_float(boxsize),
            C.c_int(nc), C.c_int(sign), _p(mesh))
        return mesh

    def assign_on_global_mesh(self, x, v, dens, rk, igrp, boxsize, nc, sign=-1, coords=(0, 0, 0)):
        mesh = np.zeros(6 * nc ** 3, np.float32)
        co = np.asarray(coords, np.int32)
        self.lib.ref_assign_on_global_mesh(
            _p(np.ascontiguousarray(x, np.float32)), _p(np.ascontiguousarray(v, np.float32)),
            _p(np.ascontiguousarray(dens, np.float32)), _p(np.ascontiguousarray(rk, np.float32)),
            _p(np.ascontiguousarray(igrp, np.int32)), C.c_int(x.shape[0]), C.c_float(boxsize),
            C.c_int(nc), C.c_int(sign), _p(co), _p(mesh))
        return mesh

    def assign_on_density_mesh(self, x, rk, igrp, boxsize, nc, sign=-1):
        mesh = np.zeros(nc ** 3, np.float32)
        self.lib.ref_assign_on_density_mesh(
            _p(np.ascontiguousarray(x, np.float32)), _p(np.ascontiguousarray(rk, np.float32)),
            _p(np.ascontiguousarray(igrp, np.int32)), C.c_int(x.shape[0]), C.c_float(boxsize),
            C.c_int(nc), C.c_int(sign), _p(mesh))
        return mesh

    def mesh_total(self, mesh, nc):
        return self.lib.ref_mesh_total(_p(np.ascontiguousarray(mesh, np.float32)), C.c_int(nc))

    def write_mesh_separate(self, base, inode, mesh, nc, boxsize):
        m = np.array(mesh, np.float32)
        self.lib.ref_write_mesh_separate(C.c_char_p(base.encode()), C.c_int(inode), _p(m),
                                         C.c_int(nc), C.c_float(boxsize))
        return m

    def read_pm_file_zip(self, filebase, redshift, inode, nc_node_dim, mesh_scale, cap,
                         shift=(0, 0, 0)):
        x, v = np.zeros((cap, 3), np.float32), np.zeros((cap, 3), np.float32)
        n, L = C.c_int(0), C.c_float(0)
        sh = np.asarray(shift, np.float32)
        rc = self.lib.ref_read_pm_file_zip(filebase.encode(), redshift.encode(), C.c_int(inode),
                                           C.c_int(nc_node_dim), C.c_int(mesh_scale), _p(sh),
                                           C.c_int(cap), _p(x), _p(v), C.byref(n), C.byref(L))
        if rc:
            raise RuntimeError("ref_read_pm_file_zip failed")
        return x[:n.value].copy(), v[:n.value].copy(), np.float32(L.value)

    def read_pm_file_xv(self, filebase, redshift, inode, cap, shift=(0, 0, 0)):
        x, v = np.zeros((cap, 3), np.float32), np.zeros((cap, 3), np.float32)
        n = C.c_int(0)
        sh = np.asarray(shift, np.float32)
        rc = self.lib.ref_read_pm_file_xv(filebase.encode(), redshift.encode(), C.c_int(inode),
                                          _p(sh), C.c_int(cap), _p(x), _p(v), C.byref(n))
        if rc:
            raise RuntimeError("ref_read_pm_file_xv failed")
        return x[:n.value].copy(), v[:n.value].copy()

    def exchange_buffer(self, x, v, boxsize, buffer_factor):
        """One-rank exchange_buffer + remove_extra_particles: (x, v, np_local)."""
        x = np.ascontiguousarray(x, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        cap = 8 * len(x) + 1024
        ox, ov = np.zeros((cap, 3), np.float32), np.zeros((cap, 3), np.float32)
        nw, nl = C.c_int(0), C.c_int(0)
        rc = self.lib.ref_exchange_buffer(_p(x), _p(v), C.c_int(len(x)), C.c_float(boxsize),
                                          C.c_float(buffer_factor), _p(ox), _p(ov), C.c_int(cap),
                                          C.byref(nw), C.byref(nl))
        if rc:
            raise RuntimeError("ref_exchange_buffer failed")
        return ox[:nw.value].copy(), ov[:nw.value].copy(), nl.value

    def write_mesh(self, filename, mesh, nc, boxsize):
        m = np.array(mesh, np.float32)
        self.lib.ref_write_mesh(C.c_char_p(filename.encode()), _p(m), C.c_int(nc),
                                C.c_float(boxsize))

    def write_fof_halos(self, filename, x, v, igrp, nhalo, boxsize):
        self.lib.ref_write_fof_halos(C.c_char_p(filename.encode()),
                                     _p(np.ascontiguousarray(x, np.float32)),
                                     _p(np.ascontiguousarray(v, np.float32)),
                                     _p(np.ascontiguousarray(igrp, np.int32)),
                                     C.c_int(len(igrp)), C.c_int(nhalo), C.c_float(boxsize))

    def group_fof(self, x, left, right, ll):
        x = np.ascontiguousarray(x, np.float32)
        igrp = np.zeros(x.shape[0], np.int32)
        ng = C.c_int(0)
        self.lib.ref_group_fof(_p(x), C.c_int(x.shape[0]), C.c_float(left), C.c_float(right),
                               C.c_float(ll), _p(igrp), C.byref(ng))
        return igrp, ng.value

    def remove_small_groups(self, igrp, ngrp):
        g = np.array(igrp, np.int32)
        nh = C.c_int(0)
        self.lib.ref_remove_small_groups(_p(g), C.c_int(g.size), C.c_int(ngrp), C.byref(nh))
        return g, nh.value

    def mark_halo_particles(self, x, left, right, halos, igrp=None):
        x = np.ascontiguousarray(x, np.float32)
        g = np.zeros(x.shape[0], np.int32) if igrp is None else np.array(igrp, np.int32)
        h = np.ascontiguousarray(halos, np.float32).reshape(-1, 5)
        nph = C.c_long(0)
        mh = C.c_double(0.0)
        self.lib.ref_mark_halo_particles(_p(x), C.c_int(x.shape[0]), C.c_float(left), C.c_float(right),
                                         _p(h), C.c_int(h.shape[0]), _p(g), C.byref(nph), C.byref(mh))
        return g, nph.value, mh.value


def canonical_groups(igrp: np.ndarray) -> np.ndarray:
    """Relabel a partition by the minimum input index of each group (label 0 and
    negative labels are kept as they are) so that two labellings compare equal
    iff they describe the same partition."""
    g = np.asarray(igrp)
    out = g.copy()
    pos = g > 0
    if not pos.any():
        return out
    idx = np.nonzero(pos)[0]
    labels = g[idx]
    order = np.lexsort((idx, labels))
    sl, si = labels[order], idx[order]
    first = np.ones(sl.size, bool)
    first[1:] = sl[1:] != sl[:-1]
    rep = np.maximum.accumulate(np.where(first, np.arange(sl.size), 0))
    out[si] = si[rep] + 1
    return out
