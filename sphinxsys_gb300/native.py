"""ctypes binding of libsphx_cuda.so (the C ABI declared in include/sphx/sphx.h).

The library is built in-tree by sphinxsys_gb300/build.py.  Loading fails loudly when it
is missing: there is no CPU fallback.  With SPHX_CHECKED_BUILD=1 in the environment the
bounds-checked build (build.py --checked) is loaded instead.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

from . import build as _build

SPHX_OK = 0
ERRORS = {1: "SPHX_ERR_INVALID_ARG", 2: "SPHX_ERR_CUDA", 3: "SPHX_ERR_CAPACITY", 4: "SPHX_ERR_OUT_OF_MEMORY",
          5: "SPHX_ERR_NOT_FOUND", 6: "SPHX_ERR_TIMEOUT", 7: "SPHX_ERR_NUMERIC", 8: "SPHX_ERR_NO_DEVICE",
          9: "SPHX_ERR_BOUNDS"}
F64, U32, F32, I32 = 0, 1, 2, 3


class SphxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class MeshDesc(C.Structure):
    _fields_ = [("dim", C.c_int), ("all_cells", C.c_int * 3), ("lower", C.c_double * 3),
                ("grid_spacing", C.c_double)]


class FluidParams(C.Structure):
    _fields_ = [("rho0", C.c_double), ("c0", C.c_double), ("h", C.c_double), ("sigma0", C.c_double),
                ("limiter_slope", C.c_double), ("acoustic_cfl", C.c_double), ("advection_cfl", C.c_double),
                ("U_ref", C.c_double)]


# name -> (restype, argtypes); every function returns int status unless stated.
_vp, _d, _i, _sz = C.c_void_p, C.c_double, C.c_int, C.c_size_t
_pd, _pu32, _pu64, _psz = C.POINTER(C.c_double), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), C.POINTER(C.c_size_t)
_pvp = C.POINTER(C.c_void_p)
SIGNATURES = {
    "sphx_last_error": (C.c_char_p, []),
    "sphx_version": (C.c_char_p, []),
    "sphx_checked_build": (C.c_int, []),
    "sphx_check_violations": (C.c_int, [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int]),
    "sphx_ctx_create": (_i, [_i, _vp, _pvp]),
    "sphx_ctx_destroy": (_i, [_vp]),
    "sphx_ctx_synchronize": (_i, [_vp]),
    "sphx_ctx_launch_count": (_i, [_vp, _pu64]),
    "sphx_ctx_stream": (_i, [_vp, _pvp]),
    "sphx_body_create": (_i, [_vp, _i, _sz, _pvp]),
    "sphx_body_destroy": (_i, [_vp]),
    "sphx_body_size": (_i, [_vp, _psz]),
    "sphx_body_register": (_i, [_vp, C.c_char_p, _i, _i]),
    "sphx_body_upload": (_i, [_vp, C.c_char_p, _i, _i, _vp, _sz]),
    "sphx_body_download": (_i, [_vp, C.c_char_p, _vp, _sz]),
    "sphx_body_upload_rows": (_i, [_vp, C.c_char_p, _vp, _sz, _sz]),
    "sphx_body_download_rows": (_i, [_vp, C.c_char_p, _vp, _sz, _sz]),
    "sphx_body_device_ptr": (_i, [_vp, C.c_char_p, _pvp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sphx_body_check_finite": (_i, [_vp, C.c_char_p, _pu64]),
    "sphx_mesh_from_bounds": (_i, [_i, _pd, _pd, _d, _i, C.POINTER(MeshDesc)]),
    "sphx_cell_list_create": (_i, [_vp, C.POINTER(MeshDesc), _sz, _pvp]),
    "sphx_cell_list_destroy": (_i, [_vp]),
    "sphx_cell_list_update": (_i, [_vp, _vp]),
    "sphx_cell_list_num_cells": (_i, [_vp, _psz]),
    "sphx_cell_list_download": (_i, [_vp, _pu32, _pu32, _sz]),
    "sphx_exclusive_scan_u32": (_i, [_vp, _vp, _vp, _sz, _pu32]),
    "sphx_exclusive_scan_u32_noalloc": (_i, [_vp, _vp, _vp, _sz, _pu32]),
    "sphx_inner_relation_create": (_i, [_vp, _vp, _d, _pvp]),
    "sphx_contact_relation_create": (_i, [_vp, _vp, _vp, _d, _i, _d, _pvp]),
    "sphx_relation_destroy": (_i, [_vp]),
    "sphx_relation_update": (_i, [_vp]),
    "sphx_relation_download": (_i, [_vp, _pu32, _pu32, _pd, _pd, _pd, _pd, _psz]),
    "sphx_lattice_number_density": (_i, [_i, _d, _d, _pd]),
    "sphx_density_summation_complex_free_surface": (_i, [_vp, _vp, C.POINTER(FluidParams)]),
    "sphx_integration_1st_half_with_wall_riemann": (_i, [_vp, _vp, C.POINTER(FluidParams), _d]),
    "sphx_integration_2nd_half_with_wall_riemann": (_i, [_vp, _vp, C.POINTER(FluidParams), _d]),
    "sphx_acoustic_time_step": (_i, [_vp, C.POINTER(FluidParams), _pd]),
    "sphx_advection_time_step": (_i, [_vp, C.POINTER(FluidParams), _pd]),
    "sphx_gravity_force": (_i, [_vp, _pd]),
    "sphx_particle_sorting": (_i, [_vp, C.POINTER(MeshDesc)]),
    "sphx_observe_quantity": (_i, [_vp, C.c_char_p, _pd]),
    "sphx_total_mechanical_energy": (_i, [_vp, _pd, _pd]),
    "sphx_upper_front_in_axis_direction": (_i, [_vp, _i, _pd, _pd, _pd]),
    "sphx_cell_list_set_periodic": (_i, [_vp, _i, _d, _d, _d]),
    "sphx_cell_list_num_entries": (_i, [_vp, _psz]),
    "sphx_periodic_bounding": (_i, [_vp, _i, _d, _d]),
    "sphx_relation_keep_distances": (_i, [_vp]),
    "sphx_density_summation_inner": (_i, [_vp, C.POINTER(FluidParams)]),
    "sphx_viscous_force_inner": (_i, [_vp, _d]),
    "sphx_transport_velocity_correction_inner": (_i, [_vp, _d]),
    "sphx_maximum_speed": (_i, [_vp, _pd]),
    "sphx_ck_density_regularization": (_i, [_vp, _vp, C.POINTER(FluidParams)]),
    "sphx_ck_advection_step_setup": (_i, [_vp]),
    "sphx_ck_update_particle_position": (_i, [_vp]),
    "sphx_ck_free_surface_indication": (_i, [_vp, _vp]),
    "sphx_ck_compression_summation": (_i, [_vp, _vp]),
    "sphx_ck_free_surface_regularization": (_i, [_vp, C.c_double]),
    "sphx_ck_linear_correction_matrix": (_i, [_vp, _vp, _d]),
    "sphx_ck_acoustic_step_1st_half": (_i, [_vp, _vp, C.POINTER(FluidParams), _d]),
    "sphx_ck_acoustic_step_2nd_half": (_i, [_vp, _vp, C.POINTER(FluidParams), _d]),
    "sphx_ck_acoustic_time_step": (_i, [_vp, C.POINTER(FluidParams), _pd]),
    "sphx_ck_advection_time_step": (_i, [_vp, C.POINTER(FluidParams), _pd]),
    "sphx_ck_observe_quantity": (_i, [_vp, C.c_char_p, _pd]),
    "sphx_mp_create": (_i, [_vp, _vp, C.POINTER(FluidParams), _pd, _pvp]),
    "sphx_mp_create_periodic": (_i, [_vp, C.POINTER(FluidParams), _pd, _pd, C.c_double, C.c_double, _pvp]),
    "sphx_mp_destroy": (_i, [_vp]),
    "sphx_mp_advection_step": (_i, [_vp, _i, C.POINTER(C.c_int), _pd, _pd]),
    "sphx_mp_download": (_i, [_vp, _vp]),
    "sphx_mp_upload": (_i, [_vp, _vp]),
    "sphx_mp_upload_host": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "sphx_mp_download_host": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "sphx_mp_set_host_rows": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "sphx_mp_conservation": (_i, [_vp, _pd]),
    "sphx_mp_upper_front": (_i, [_vp, _i, _pd, _pd, _pd]),
    "sphx_mp_check_state": (_i, [_vp, _pu64, _pu64]),
    "sphx_mp_set_tuning": (_i, [_vp, _i, _i]),
    "sphx_mp_set_tile": (_i, [_vp, _i, _i, _i]),
    "sphx_mp_get_tuning": (_i, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sphx_mp_set_profiling": (_i, [_vp, _i]),
    "sphx_mp_autotune": (_i, [_vp, _i, C.POINTER(C.c_int), C.POINTER(C.c_int), _pd]),
    "sphx_mp_kernel_times": (_i, [_vp, _pd]),
    "sphx_mp_list_sizes": (_i, [_vp, _pu64]),
    "sphx_batch_create": (_i, [_vp, _i, _i, _vp, _pvp]),
    "sphx_batch_destroy": (_i, [_vp]),
    "sphx_batch_advection_step": (_i, [_vp, _i, C.POINTER(C.c_int), _pd]),
    "sphx_batch_set_tuning": (_i, [_vp, _i]),
    "sphx_batch_set_substep_cap": (_i, [_vp, _i]),
    "sphx_batch_graph_launches": (_i, [_vp, _pu64]),
    "sphx_batch_download": (_i, [_vp, _i, _pd, _pd, _pd, _pd]),
    "sphx_batch_size": (_i, [_vp, _psz, _psz]),
}

_lib: Optional[C.CDLL] = None


def checked_requested() -> bool:
    return os.environ.get("SPHX_CHECKED_BUILD", "0") not in ("", "0")


def library_path() -> str:
    return _build.LIB_CHECK if checked_requested() else _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Loads libsphx_cuda.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build it with sphinxsys_gb300/build.py "
                               "(there is no CPU fallback)")
        _build.build(checked=checked_requested())
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != SPHX_OK:
        msg = load().sphx_last_error()
        raise SphxError(status, msg.decode() if msg else "")


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def check_violations(reset: bool = True) -> tuple:
    """(count, site, value) of the bounds-checked build's failed index tests since the last
    reset, the site and value of the first one (count 0 in other builds); synchronises."""
    c, f = C.c_uint64(), C.c_uint64()
    st = load().sphx_check_violations(C.byref(c), C.byref(f), int(reset))
    if st not in (SPHX_OK, 9):
        check(st)
    return c.value, f.value >> 48, f.value & ((1 << 48) - 1)
