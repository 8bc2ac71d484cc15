"""ctypes binding of libasmooth_gb300.so (the C ABI in include/asmooth_gb300.h).

The library is loaded from this package directory only; there is no CPU
fallback: importing the binding without the built library raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libasmooth_gb300.so")

# every symbol include/asmooth_gb300.h declares, with (restype, argtypes)
_vp, _i, _f, _d = C.c_void_p, C.c_int, C.c_float, C.c_double
_ip, _fp, _dp, _lp = C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_long)
SIGNATURES = {
    "asg_create": (_i, [C.POINTER(_vp), _i]),
    "asg_destroy": (None, [_vp]),
    "asg_strerror": (C.c_char_p, [_i]),
    "asg_last_error": (C.c_char_p, [_vp]),
    "asg_abi_version": (_i, []),
    "asg_host_alloc": (_i, [C.c_size_t, C.POINTER(_vp)]),
    "asg_host_free": (_i, [_vp]),
    "asg_neighbor_search": (_i, [_vp, _vp, _i, _f, _f]),
    "asg_assign_on_mesh": (_i, [_vp, _vp, _i, _f, _i, _i, _vp, _vp]),
    "asg_assign_on_meshes": (_i, [_vp, _vp, _i, _f, _vp, _i, _i, _i, _vp, _vp, _vp]),
    "asg_assign_on_density_mesh": (_i, [_vp, _vp, _i, _f, _i, _i, _vp]),
    "asg_normalise_mesh": (_i, [_vp, _vp, _i, _f]),
    "asg_group_fof": (_i, [_vp, _vp, _i, _f, _f, _f, _ip]),
    "asg_remove_small_groups": (_i, [_vp, _vp, _i, _i, _ip]),
    "asg_mark_halo_particles": (_i, [_vp, _vp, _i, _vp, _i, _f, _f, _lp, _dp]),
    "asg_smooth": (_i, [_vp, _vp, _i, _f, _f, _f, _vp, _i, _vp, _i, _i, _vp, _vp, _lp, _dp]),
    "asg_write_mesh_separate": (_i, [_vp, C.c_char_p, _i, _vp, _i, _f]),
    "asg_write_mesh_device": (_i, [_vp, _i, C.c_char_p, _i]),
    "asg_write_mesh": (_i, [C.c_char_p, _vp, _i, _f]),
    "asg_fof_halos": (_i, [_vp, _vp, _i, _i, _f, _vp, _ip]),
    "asg_write_fof_halos": (_i, [_vp, C.c_char_p, _vp, _i, _i, _f]),
    "asg_run_fof_halos": (_i, [_vp, _i, _f, _vp, _ip]),
    "asg_load_periodic_cube": (_i, [_vp, _vp, _i, _f, _f, _ip, _ip]),
    "asg_load_periodic_cube_device": (_i, [_vp, _vp, _vp, _i, _f, _f, _ip, _ip]),
    "asg_decode_xv": (_i, [_vp, _vp, _i, _vp]),
    "asg_decode_zip": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _i, _i, _i, _f, _vp]),
    "asg_read_pm_file_xv": (_i, [_vp, C.c_char_p, C.c_char_p, _i, _vp, _ip]),
    "asg_read_pm_file_zip": (_i, [_vp, C.c_char_p, C.c_char_p, _i, _i, _i, _vp, _ip, _fp]),
    "asg_copy_decoded": (_i, [_vp, _vp]),
    "asg_load_decoded_periodic": (_i, [_vp, _f, _f, _ip, _ip]),
    "asg_batch_create": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _i, _i, C.POINTER(_vp)]),
    "asg_batch_destroy": (None, [_vp]),
    "asg_batch_set_item": (_i, [_vp, _i, _vp, _vp, _i]),
    "asg_batch_set_item_quantised": (_i, [_vp, _i, _vp, _vp, _vp, _f, _i, _i]),
    "asg_batch_tune": (_i, [_vp, _ip, _ip]),
    "asg_batch_config": (_i, [_vp, _ip, _ip, _ip, _ip]),
    "asg_batch_set_streams": (_i, [_vp, _i]),
    "asg_batch_run": (_i, [_vp]),
    "asg_batch_stats": (_i, [_vp, _dp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "asg_batch_get": (_i, [_vp, _i, _vp, _vp, _vp, _vp]),
    "asg_load_particles": (_i, [_vp, _vp, _i, _f, _f]),
    "asg_load_particles_device": (_i, [_vp, _vp, _vp, _vp, _vp, _i, _f, _f]),
    "asg_load_particles_quantised": (_i, [_vp, _vp, _vp, _vp, _i, _f, _f, _f, _i]),
    "asg_load_particles_quantised_device": (_i, [_vp, _vp, _vp, _vp, _i, _f, _f, _f, _i]),
    "asg_smooth_quantised": (_i, [_vp, _vp, _vp, _vp, _i, _f, _f, _f, _i, _f, _vp, _i, _i,
                                  _vp, _vp, _vp, _vp]),
    "asg_run_neighbor_search": (_i, [_vp]),
    "asg_run_mark_halos": (_i, [_vp, _vp, _i, _lp, _dp]),
    "asg_run_fof": (_i, [_vp, _f, _ip]),
    "asg_run_remove_small_groups": (_i, [_vp, _i, _ip]),
    "asg_run_deposit": (_i, [_vp, _f, _vp, _i, _i, _i, _vp, _i, _vp]),
    "asg_run_normalise": (_i, [_vp, _i]),
    "asg_mesh_device": (_vp, [_vp, _i]),
    "asg_copy_mesh": (_i, [_vp, _i, _vp]),
    "asg_store_particles": (_i, [_vp, _vp]),
    "asg_store_fields_device": (_i, [_vp, _vp, _vp, _vp]),
    "asg_get_knn": (_i, [_vp, _vp, _vp]),
    "asg_stream": (_vp, [_vp]),
    "asg_kernel_launches": (C.c_longlong, [_vp]),
    "asg_set_timing": (_i, [_vp, _i]),
    "asg_phase_ms": (_i, [_vp, _vp]),
    "asg_phase_name": (C.c_char_p, [_i]),
    "asg_measure_fp32_peak": (_i, [_vp, _dp]),
    "asg_deposit_stats": (_i, [_vp, _vp, _vp, _vp]),
    "asg_neighbor_search_noalloc": (_i, [_vp, _i, _f, _f, _vp, _vp, _vp]),
}
NPHASES = 10

_LIB = None


def load() -> C.CDLL:
    """Load the in-tree library; raise if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "or `python -m asmooth_gb300.build` (no CPU fallback exists)")
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib
