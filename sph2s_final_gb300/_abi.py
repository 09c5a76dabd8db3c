"""ctypes binding of include/sph2s.h (libsph2s.so, built in-tree).

There is no fallback: if the CUDA library is missing or fails to load, every
call raises.  Build it with `python -m sph2s_final_gb300.build`.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libsph2s.so"

SPH_OK = 0
SPH_E_INVALID = 1
SPH_E_CAPACITY = 2
SPH_E_CUDA = 3
SPH_E_TIMEOUT = 4
SPH_E_IO = 5
SPH_ORDER_SORTED = 0
SPH_ORDER_BY_ID = 1

_STATUS = {1: "SPH_E_INVALID", 2: "SPH_E_CAPACITY", 3: "SPH_E_CUDA", 4: "SPH_E_TIMEOUT",
           5: "SPH_E_IO"}


class SphError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


class sph_grid(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("dims", C.c_int32 * 3), ("spacing", C.c_float)]


class sph_config(C.Structure):
    _fields_ = [
        ("effective_radius", C.c_float),
        ("fluid_particle_mass", C.c_float),
        ("boundary_particle_mass", C.c_float),
        ("rest_density", C.c_float),
        ("bulk_modulus", C.c_float),
        ("viscosity", C.c_float),
        ("speed_sound", C.c_float),
        ("tension_coefficient", C.c_float),
        ("xsph_coeff", C.c_float),
        ("grid", sph_grid),
    ]


class sph_config2(C.Structure):
    _fields_ = [
        ("effective_radius", C.c_float * 2),
        ("fluid_particle_mass", C.c_float * 2),
        ("boundary_particle_mass", C.c_float),
        ("rest_density", C.c_float),
        ("bulk_modulus", C.c_float),
        ("viscosity", C.c_float),
        ("speed_sound", C.c_float),
        ("tension_coefficient", C.c_float),
        ("blend_increment", C.c_float),
        ("grid", sph_grid * 2),
        ("refine_axis", C.c_int32),
        ("refine_lo", C.c_float),
        ("refine_hi", C.c_float),
        ("mode", C.c_int32),
        ("split_trigger", C.c_int32),
        ("surface_density", C.c_float),
    ]


class sph_scene_desc(C.Structure):
    _fields_ = [
        ("fluid_xyz", C.POINTER(C.c_float)),
        ("n_fluid", C.c_uint32),
        ("boundary_xyz", C.POINTER(C.c_float)),
        ("n_boundary", C.c_uint32),
        ("velocity_xyz", C.POINTER(C.c_float)),
        ("config", sph_config),
    ]


_f = C.POINTER(C.c_float)
_u = C.POINTER(C.c_uint32)
_vp = C.c_void_p

# name -> (restype, argtypes)
SIGNATURES = {
    "sph_make_grid": (C.c_int, [_f, _f, C.c_float, C.POINTER(sph_grid)]),
    "sph_grid_num_cells": (C.c_uint32, [C.POINTER(sph_grid)]),
    "sph_make_configuration": (C.c_int, [_f, _f, C.c_float, C.c_uint32, C.c_uint32, C.c_float,
                                         C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                         C.POINTER(sph_config)]),
    "sph_particle_box": (C.c_int, [C.POINTER(sph_grid), _f, C.c_uint32, _u]),
    "sph_particle_box_canvas": (C.c_int, [C.POINTER(sph_grid), C.c_int32, _f, C.c_uint32, _u]),
    "sph_create": (C.c_int, [C.POINTER(sph_config), _f, C.c_uint32, _f, C.c_uint32, _f,
                             C.POINTER(_vp)]),
    "sph_advance": (C.c_int, [_vp, C.c_float, C.c_int32]),
    "sph_sync": (C.c_int, [_vp]),
    "sph_get_positions": (C.c_int, [_vp, _f, C.c_int32]),
    "sph_get_positions_async": (C.c_int, [_vp, _f, C.c_int32]),
    "sph_get_velocities": (C.c_int, [_vp, _f, C.c_int32]),
    "sph_get_densities": (C.c_int, [_vp, _f, C.c_int32]),
    "sph_get_positions_device": (C.c_int, [_vp, C.c_void_p, C.c_int32]),
    "sph_get_velocities_device": (C.c_int, [_vp, C.c_void_p, C.c_int32]),
    "sph_get_densities_device": (C.c_int, [_vp, C.c_void_p, C.c_int32]),
    "sph2_get_positions_device": (C.c_int, [_vp, C.c_int32, C.c_void_p]),
    "sph2_get_states_device": (C.c_int, [_vp, C.c_int32, C.c_void_p]),
    "sph_get_ids": (C.c_int, [_vp, _u]),
    "sph_set_velocities": (C.c_int, [_vp, _f, C.c_int32]),
    "sph_counts": (C.c_int, [_vp, _u, _u]),
    "sph_stream": (C.c_void_p, [_vp]),
    "sph_destroy": (C.c_int, [_vp]),
    "sph_debug_step_fields": (C.c_int, [_vp, _u, _u, _u, _u, _u, _u, _f, _f]),
    "sph_profile_phases": (C.c_int, [_vp, C.c_float, C.c_int32, _f]),
    "sph_debug_force_lookback_timeout": (C.c_int, [_vp, C.c_int32]),
    "sph_debug_sort_mode": (C.c_int, [_vp, C.c_int32]),
    "sph_rollout_forward": (C.c_int, [_vp, _f, C.c_float, C.c_float, C.c_int32, C.c_int32]),
    "sph_rollout_density_loss": (C.c_int, [_vp, C.POINTER(sph_grid), _f, _f,
                                           C.POINTER(C.c_double)]),
    "sph_rollout_backward": (C.c_int, [_vp, _f, _f, C.POINTER(C.c_double)]),
    "sph_make_configuration2": (C.c_int, [_f, _f, C.c_float, C.c_uint32, C.c_uint32, C.c_float,
                                          C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                          C.POINTER(sph_config2)]),
    "sph2_create": (C.c_int, [C.POINTER(sph_config2), _f, C.c_uint32, _f, C.c_uint32, _f,
                              C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(_vp)]),
    "sph2_advance": (C.c_int, [_vp, C.c_float, C.c_int32]),
    "sph2_counts": (C.c_int, [_vp, _u, _u, _u, _u]),
    "sph2_last_stats": (C.c_int, [_vp, _u]),
    "sph2_next_ids": (C.c_int, [_vp, _u, _u]),
    "sph2_get_state": (C.c_int, [_vp, C.c_int32, _f, _f, _f, C.POINTER(C.c_int32), _u, _u]),
    "sph2_debug_step_fields": (C.c_int, [_vp, C.c_int32, _u, _f, _f, _u, _u, _u]),
    "sph2_destroy": (C.c_int, [_vp]),
    "sph2_set_color_output": (C.c_int, [_vp, C.c_int32]),
    "sph2_get_colors": (C.c_int, [_vp, C.c_int32, _f, _u, _u]),
    "sphb_create": (C.c_int, [C.POINTER(sph_scene_desc), C.c_uint32, C.POINTER(_vp)]),
    "sphb_advance": (C.c_int, [_vp, C.c_float, C.c_int32]),
    "sphb_sync": (C.c_int, [_vp]),
    "sphb_stream": (C.c_void_p, [_vp]),
    "sphb_counts": (C.c_int, [_vp, _u, _u, _u]),
    "sphb_get_scene": (C.c_int, [_vp, C.c_uint32, _f, _f, _f, C.c_int32]),
    "sphb_autotune": (C.c_int, [_vp, C.c_float, C.POINTER(C.c_int32)]),
    "sphb_destroy": (C.c_int, [_vp]),
    "sphb_rollout_forward": (C.c_int, [_vp, _f, _f, C.c_float, C.c_int32, C.c_int32]),
    "sphb_rollout_density_loss": (C.c_int, [_vp, C.POINTER(sph_grid), _f, _f,
                                            C.POINTER(C.c_double)]),
    "sphb_rollout_backward": (C.c_int, [_vp, _f, _f, C.POINTER(C.c_double)]),
    "sph_sort_pairs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32,
                                 C.c_int32, C.c_void_p]),
    "sph_sort_pairs_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_uint32, C.c_int32, C.c_void_p]),
    "sph_sort_keys_coherent": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_uint32, C.c_int32, C.c_void_p]),
    "sph_set_integrator": (C.c_int, [_vp, C.c_int32]),
    "sph_step_count": (C.c_int, [_vp, C.POINTER(C.c_uint64)]),
    "sph_save_state": (C.c_int, [_vp, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "sph_create_from_state": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(_vp)]),
    "sph_write_frame": (C.c_int, [_vp, C.c_char_p, C.c_uint32, C.c_int32]),
    "sph2_step_count": (C.c_int, [_vp, C.POINTER(C.c_uint64)]),
    "sph2_save_state": (C.c_int, [_vp, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint64)]),
    "sph2_create_from_state": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(_vp)]),
    "sph2_write_frame": (C.c_int, [_vp, C.c_char_p, C.c_uint32, C.c_int32]),
    "sph_last_error": (C.c_char_p, []),
}

_lib = None


def lib() -> C.CDLL:
    """Loads libsph2s.so once and declares every exported signature."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH.name} is not built; run `python -m sph2s_final_gb300.build` "
                "(there is no CPU fallback)")
        l = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(rc: int) -> None:
    if rc != SPH_OK:
        raise SphError(rc, lib().sph_last_error().decode(errors="replace"))


def fptr(a):
    return a.ctypes.data_as(_f) if a is not None else None


def uptr(a):
    return a.ctypes.data_as(_u) if a is not None else None
