"""CPU tests of the C-ABI library: it builds, loads, exports every symbol the
public header declares, and its host-only entry points behave; no kernel is
launched."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "asmooth_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(asg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from asmooth_gb300 import build as B
    from asmooth_gb300 import _lib

    B.build()
    return _lib.load()


def test_header_declares_the_entry_points():
    syms = declared_symbols()
    for s in ("asg_create", "asg_neighbor_search", "asg_assign_on_mesh", "asg_assign_on_meshes",
              "asg_group_fof", "asg_remove_small_groups", "asg_mark_halo_particles", "asg_smooth",
              "asg_normalise_mesh", "asg_assign_on_density_mesh"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    from asmooth_gb300 import _lib

    for s in declared_symbols():
        assert hasattr(lib, s), s
        assert s in _lib.SIGNATURES, f"{s} has no ctypes signature"


def test_host_only_entry_points(lib):
    assert lib.asg_abi_version() == 2
    assert lib.asg_strerror(0) == b"ok"
    assert b"33" in lib.asg_strerror(-4)
    assert lib.asg_strerror(12345) == b"unknown status"
    assert lib.asg_create(None, 0) == -1  # null out-pointer is rejected before any CUDA call
    assert lib.asg_last_error(None) == b"no context"


def test_host_alloc_argument_checks(lib):
    import ctypes as C

    assert lib.asg_host_alloc(16, None) == -1  # null out-pointer
    out = C.c_void_p(1)
    assert lib.asg_host_alloc(0, C.byref(out)) == -1 and not out.value  # zero bytes; out cleared
    assert lib.asg_host_free(None) == 0  # null is a no-op
    junk = C.create_string_buffer(64)
    assert lib.asg_host_free(C.cast(junk, C.c_void_p)) == -1  # not a block of asg_host_alloc


def test_particle_record_layout():
    from asmooth_gb300 import api

    assert api.PARTICLE_DTYPE.itemsize == 36 and api.HALO_DTYPE.itemsize == 20
    p = api.make_particles([[1, 2, 3]], v=[[4, 5, 6]], dens=[7], rk=[8], igrp=[9])
    raw = p.tobytes()
    vals = C.cast(C.c_char_p(raw), C.POINTER(C.c_float))
    assert [vals[i] for i in range(8)] == [1, 2, 3, 4, 5, 6, 7, 8]
    assert C.cast(C.c_char_p(raw), C.POINTER(C.c_int))[8] == 9


def test_binding_fails_loudly_without_library(tmp_path, monkeypatch):
    from asmooth_gb300 import _lib

    monkeypatch.setattr(_lib, "_LIB", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError):
        _lib.load()
