"""ctypes declarations of include/xpbd.h and the library loader.

The binding a maintainer of the reference would add to call this library
from Python is exactly this file plus vkxpbd/__init__.py.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libxpbd_gb300.so")


class Config(C.Structure):
    """struct xpbd_config (include/xpbd.h)."""

    _fields_ = [
        ("dt", C.c_float), ("substeps", C.c_int32), ("iterations", C.c_int32),
        ("particle_v_max", C.c_float), ("soft_contact_mu", C.c_float), ("shape_material_mu", C.c_float),
        ("soft_contact_relaxation", C.c_float), ("particle_adhesion", C.c_float), ("particle_mu", C.c_float),
        ("particle_cohesion", C.c_float), ("particle_max_radius", C.c_float), ("search_radius", C.c_float),
        ("soft_contact_margin", C.c_float), ("enable_restitution", C.c_int32),
        ("soft_contact_restitution", C.c_float), ("has_ground_plane", C.c_int32),
        ("ground_plane_altitude", C.c_float), ("gravity", C.c_float * 3), ("shader_dir", C.c_char * 256),
        ("device_index", C.c_int32), ("compat_mode", C.c_int32), ("enable_validation", C.c_int32),
        ("enable_diagnostics", C.c_int32), ("enable_profile", C.c_int32), ("max_diag_pairs", C.c_uint32),
        ("substep_batch_size", C.c_int32),
    ]


class PairRecord(C.Structure):
    """struct xpbd_pair_record (vkx::GPUPairRecord, src/scene.h:43-64)."""

    _fields_ = [
        ("i", C.c_uint32), ("j", C.c_uint32), ("dist", C.c_float), ("err", C.c_float),
        ("normal", C.c_float * 3), ("vrel", C.c_float * 3), ("vn", C.c_float), ("vt_len", C.c_float),
        ("denom", C.c_float), ("lambda_n", C.c_float), ("lambda_f", C.c_float), ("delta_i", C.c_float * 3),
        ("iter_index", C.c_uint32), ("pad0", C.c_uint32),
    ]


class BodyParams(C.Structure):
    """struct xpbd_body_params (include/xpbd.h)."""

    _fields_ = [
        ("angular_damping", C.c_float), ("rigid_contact_margin", C.c_float),
        ("rigid_contact_relaxation", C.c_float), ("rigid_contact_con_weighting", C.c_int32),
        ("rigid_mu_torsional", C.c_float), ("rigid_mu_rolling", C.c_float),
        ("particle_contact_con_weighting", C.c_int32),
    ]


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)
_U = C.POINTER(C.c_uint32)
_Z = C.c_size_t

# name -> (restype, argtypes); every symbol include/xpbd.h declares
SIGNATURES = {
    "xpbd_last_error": (C.c_char_p, []),
    "xpbd_abi_version": (C.c_int, []),
    "xpbd_config_default": (None, [C.POINTER(Config)]),
    "xpbd_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "xpbd_device_name": (C.c_int, [C.c_int, C.c_char_p, _Z]),
    "xpbd_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "xpbd_destroy": (C.c_int, [_P]),
    "xpbd_init": (C.c_int, [_P, C.POINTER(Config), _Z, _Z]),
    "xpbd_add_mesh": (C.c_int, [_P, _F, _Z, _U, _Z, C.c_float, _F, C.c_int]),
    "xpbd_finalize_meshes": (C.c_int, [_P]),
    "xpbd_set_particles": (C.c_int, [_P, _F, _F, _F, _F, _I, _Z]),
    "xpbd_update_mesh": (C.c_int, [_P, _Z, _F, _Z, _F]),
    "xpbd_step": (C.c_int, [_P, C.c_float, C.c_int, C.c_int]),
    "xpbd_collide_only": (C.c_int, [_P]),
    "xpbd_step_solve_only": (C.c_int, [_P, C.c_float, C.c_int, C.c_int]),
    "xpbd_get_positions": (C.c_int, [_P, _F, _Z]),
    "xpbd_get_velocities": (C.c_int, [_P, _F, _Z]),
    "xpbd_particle_count": (_Z, [_P]),
    "xpbd_mesh_count": (_Z, [_P]),
    "xpbd_last_contact_count": (C.c_int, [_P]),
    "xpbd_get_contacts": (C.c_int, [_P, _I, _I, _F, _F, _F]),
    "xpbd_set_contact_data": (C.c_int, [_P, _I, _I, _F, _F, C.c_int]),
    "xpbd_get_sorted_cells": (C.c_int, [_P, _U, _Z]),
    "xpbd_get_sorted_point_ids": (C.c_int, [_P, _U, _Z]),
    "xpbd_get_cell_starts": (C.c_int, [_P, _I, _Z]),
    "xpbd_get_cell_ends": (C.c_int, [_P, _I, _Z]),
    "xpbd_get_deltas": (C.c_int, [_P, _F, _Z]),
    "xpbd_get_mesh_bvh": (C.c_int, [_P, _Z, _F, _F, _Z, C.POINTER(_Z)]),
    "xpbd_get_diag_pair_count": (C.c_int, [_P, _U]),
    "xpbd_get_diag_overflow_count": (C.c_int, [_P, _U]),
    "xpbd_reset_diag_buffers": (C.c_int, [_P]),
    "xpbd_get_diag_pairs": (C.c_int, [_P, C.c_void_p, _Z, C.POINTER(_Z)]),
    "xpbd_get_aux_diag": (C.c_int, [_P, C.c_int, C.c_void_p, _Z, C.POINTER(_Z)]),
    "xpbd_print_profiler_summary": (C.c_int, [_P]),
    "xpbd_get_status": (C.c_int, [_P, _U]),
    "xpbd_debug_lookback_hold": (C.c_int, [C.c_int64, C.c_uint64]),
    "xpbd_step_async": (C.c_int, [_P, C.c_float, C.c_int, C.c_int]),
    "xpbd_sync": (C.c_int, [_P]),
    "xpbd_stream": (C.c_void_p, [_P]),
    "xpbd_set_profiling": (C.c_int, [_P, C.c_int]),
    "xpbd_get_stage_times": (C.c_int, [_P, C.POINTER(C.c_double), _Z, C.POINTER(_Z), C.POINTER(C.c_uint64)]),
    "xpbd_reset_stage_times": (C.c_int, [_P]),
    "xpbd_stage_name": (C.c_char_p, [C.c_int]),
    "xpbd_get_frame_stats": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "xpbd_sort_keys_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, _Z, C.c_int, C.c_void_p]),
    "xpbd_sort_keys_noalloc_status": (C.c_int, []),
    "xpbd_body_params_default": (None, [C.POINTER(BodyParams)]),
    "xpbd_set_body_params": (C.c_int, [_P, C.POINTER(BodyParams)]),
    "xpbd_set_bodies": (C.c_int, [_P, _F, _F, _F, _F, _F, _F, _I, _Z]),
    "xpbd_set_body_scenes": (C.c_int, [_P, _I, _Z]),
    "xpbd_get_bodies": (C.c_int, [_P, _F, _F, _Z]),
    "xpbd_update_config": (C.c_int, [_P, C.POINTER(Config)]),
    "xpbd_autotune": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "xpbd_set_sort_variant": (C.c_int, [_P, C.c_int, C.c_int]),
    "xpbd_set_solve_split": (C.c_int, [_P, C.c_int]),
    "xpbd_get_kernels_launched": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "xpbd_get_solve_split": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "xpbd_set_solve_form": (C.c_int, [_P, C.c_int]),
    "xpbd_get_solve_form": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "xpbd_record_start": (C.c_int, [_P, C.c_char_p, C.c_int]),
    "xpbd_record_stop": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "xpbd_rollout": (C.c_int, [_P, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int]),
    "xpbd_rollout_backward": (C.c_int, [_P, _F, _F, _F, _F, _F, C.POINTER(C.c_double)]),
    "xpbd_batch_init": (C.c_int, [_P, C.POINTER(Config), C.POINTER(C.c_size_t), _Z, _Z]),
    "xpbd_batch_scene_count": (_Z, [_P]),
    "xpbd_batch_scene_offsets": (C.c_int, [_P, C.POINTER(C.c_size_t), _Z]),
}

_lib = None


def load() -> C.CDLL:
    """Load libxpbd_gb300.so, building it first when it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    try:
        from . import build as _build

        _build.build_library()
    except Exception as e:  # no toolchain: fall through to loading a prebuilt library
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"vkxpbd: libxpbd_gb300.so is missing and could not be built: {e}") from e
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.xpbd_abi_version() != 1:
        raise ImportError("vkxpbd: libxpbd_gb300.so ABI version mismatch")
    _lib = lib
    return lib
