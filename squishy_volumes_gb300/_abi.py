"""ctypes view of the C ABI in include/squishy_volumes_cuda.h.

The shared library is the product; this module only declares its structs and
signatures.  Loading fails loudly when the library has not been built: there
is no fallback implementation.
"""

from __future__ import annotations

import ctypes as ct
import os
from pathlib import Path

from . import build as _build

u32p = ct.POINTER(ct.c_uint32)
i32p = ct.POINTER(ct.c_int32)
f32p = ct.POINTER(ct.c_float)

SV_IS_SOLID = 1 << 0
SV_IS_FLUID = 1 << 1
SV_USE_VISCOSITY = 1 << 2
SV_USE_SAND_ALPHA = 1 << 3
SV_HAS_GOAL = 1 << 4
SV_TOMBSTONED = 1 << 5
SV_FAILED = 1 << 6

SV_STATUS_CAPACITY_EXCEEDED = 1 << 0
SV_STATUS_PARTICLE_INVERTED = 1 << 3
SV_STATUS_CANCELED = 1 << 8
SV_STATUS_SAND_INVALID_MU = 1 << 11

SV_MODEL_REFERENCE = 0
SV_MODEL_FIXED_COROTATED = 1
SV_MODEL_SNOW = 2


class SvConsts(ct.Structure):
    _fields_ = [
        ("grid_node_size", ct.c_float),
        ("domain_min", ct.c_float * 3),
        ("domain_max", ct.c_float * 3),
        ("ground_mode", ct.c_int32),
        ("ground_axis", ct.c_int32),
        ("ground_height", ct.c_float),
        ("position_form", ct.c_uint32),
        ("svd_fp64_policy", ct.c_uint32),
        ("block_capacity", ct.c_uint64),
        ("sort_interval", ct.c_uint32),
        ("host_transfer", ct.c_uint32),
        ("deterministic_p2g", ct.c_uint32),
        ("reserved", ct.c_uint32 * 3),
    ]


class SvParticles(ct.Structure):
    _fields_ = [
        ("n", ct.c_uint64),
        ("flags", u32p),
        ("positions", f32p),
        ("position_gradients", f32p),
        ("velocities", f32p),
        ("velocity_gradients", f32p),
        ("elastic_energies", f32p),
        ("collider_bits", u32p),
        ("mass", f32p),
        ("initial_volume", f32p),
        ("viscosity_dynamic", f32p),
        ("viscosity_bulk", f32p),
        ("mu", f32p),
        ("lambda_", f32p),
        ("sand_alpha", f32p),
        ("exponent", i32p),
        ("bulk_modulus", f32p),
        ("model", u32p),
        ("hardening", f32p),
        ("crit_compression", f32p),
        ("crit_stretch", f32p),
        ("plastic_j", f32p),
    ]


class SvStats(ct.Structure):
    _fields_ = [
        ("particles", ct.c_uint64),
        ("live_particles", ct.c_uint64),
        ("particle_blocks", ct.c_uint64),
        ("grid_blocks", ct.c_uint64),
        ("fp64_svd", ct.c_uint64),
        ("substeps", ct.c_uint64),
        ("device_bytes", ct.c_uint64),
        ("kernel_launches", ct.c_uint64),
        ("sorts", ct.c_uint64),
        ("sort_interval", ct.c_uint64),
        ("tile_misses", ct.c_uint64),
        ("graph_replays", ct.c_uint64),
        ("cta_per_sm", ct.c_uint64),
        ("closure_learned", ct.c_uint64),
        ("closure_fallbacks", ct.c_uint64),
        ("closure_mode", ct.c_uint64),
        ("adaptive_misses", ct.c_uint64),
        ("adaptive_split", ct.c_uint64),
        ("grid_mass", ct.c_double),
        ("grid_momentum", ct.c_double * 3),
        ("pass_ns", ct.c_uint64),
        ("pass_count", ct.c_uint64),
    ]


class SvFrameInput(ct.Structure):
    _fields_ = [
        ("frames_per_second", ct.c_uint32),
        ("frame", ct.c_uint32),
        ("has_b", ct.c_uint32),
        ("gravity_a", ct.c_float * 3),
        ("gravity_b", ct.c_float * 3),
        ("goal_flags_a", u32p),
        ("goal_flags_b", u32p),
        ("goal_positions_a", f32p),
        ("goal_positions_b", f32p),
        ("n_vertices", ct.c_uint32),
        ("n_triangles", ct.c_uint32),
        ("triangles", u32p),
        ("triangle_collider", u32p),
        ("vertex_positions_a", f32p),
        ("vertex_positions_b", f32p),
        ("friction_a", f32p),
        ("friction_b", f32p),
        ("damping_a", f32p),
        ("damping_b", f32p),
        ("leaf_size", ct.c_float),
    ]


class SvFrame(ct.Structure):
    _fields_ = [
        ("time", ct.c_double),
        ("n", ct.c_uint64),
        ("flags", u32p),
        ("mass", f32p),
        ("initial_volume", f32p),
        ("viscosity_dynamic", f32p),
        ("viscosity_bulk", f32p),
        ("mu", f32p),
        ("lambda_", f32p),
        ("sand_alpha", f32p),
        ("exponent", i32p),
        ("bulk_modulus", f32p),
        ("elastic_energies", f32p),
        ("collider_bits", u32p),
        ("positions", f32p),
        ("position_gradients", f32p),
        ("velocities", f32p),
        ("velocity_gradients", f32p),
        ("initial_positions", f32p),
        ("has_grid", ct.c_uint32),
        ("n_nodes", ct.c_uint64),
        ("node_ids", i32p),
        ("node_collider_bits", u32p),
        ("node_masses", f32p),
        ("node_velocities", f32p),
    ]


_SIGNATURES = {
    "sv_frame_write": (ct.c_int, [ct.c_char_p, ct.POINTER(SvFrame), ct.c_char_p, ct.POINTER(ct.c_uint64)]),
    "sv_frame_read": (ct.c_int, [ct.c_char_p, ct.c_char_p, ct.POINTER(SvFrame)]),
    "sv_cache_open": (ct.c_int, [ct.c_char_p, ct.c_char_p, ct.POINTER(SvFrame), ct.c_uint32, ct.c_uint32,
                                 ct.POINTER(ct.c_void_p)]),
    "sv_cache_store": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_int]),
    "sv_cache_store_frame": (ct.c_int, [ct.c_void_p, ct.POINTER(SvFrame)]),
    "sv_cache_check": (ct.c_int, [ct.c_void_p]),
    "sv_cache_flush": (ct.c_int, [ct.c_void_p]),
    "sv_cache_info": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_uint64), ct.POINTER(ct.c_uint64)]),
    "sv_cache_close": (ct.c_int, [ct.c_void_p]),
    "sv_create": (ct.c_int, [ct.POINTER(SvConsts), ct.POINTER(SvParticles), ct.POINTER(ct.c_void_p)]),
    "sv_step": (
        ct.c_int,
        [ct.c_void_p, ct.c_uint32, ct.c_float, f32p, ct.POINTER(ct.c_int32), u32p, u32p],
    ),
    "sv_download": (ct.c_int, [ct.c_void_p, ct.POINTER(SvParticles)]),
    "sv_download_grid": (ct.c_int, [ct.c_void_p, i32p, f32p, f32p, ct.c_uint64, ct.POINTER(ct.c_uint64)]),
    "sv_destroy": (None, [ct.c_void_p]),
    "sv_create_batched": (ct.c_int, [ct.POINTER(SvConsts), ct.POINTER(SvParticles), ct.c_uint32,
                                     ct.POINTER(ct.c_void_p)]),
    "sv_scene_count": (ct.c_uint32, [ct.c_void_p]),
    "sv_download_scene": (ct.c_int, [ct.c_void_p, ct.c_uint32, ct.POINTER(SvParticles)]),
    "sv_last_error_string": (ct.c_char_p, []),
    "sv_p2g_only": (ct.c_int, [ct.c_void_p, ct.c_float, f32p]),
    "sv_binning": (ct.c_int, [ct.c_void_p, u32p, u32p, u32p]),
    "sv_grid_layout": (ct.c_int, [ct.c_void_p, i32p, i32p]),
    "sv_sort_pairs": (ct.c_int, [u32p, u32p, ct.c_uint64]),
    "sv_get_stats": (ct.c_int, [ct.c_void_p, ct.POINTER(SvStats)]),
    "sv_set_stream": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "sv_set_graphs": (ct.c_int, [ct.c_void_p, ct.c_int]),
    "sv_set_host_transfer": (ct.c_int, [ct.c_void_p, ct.c_uint32, u32p]),
    "sv_prepare_host": (ct.c_int, [ct.POINTER(ct.c_void_p), ct.POINTER(ct.c_uint64), ct.c_uint32]),
    "sv_step_adaptive": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_double), ct.c_double, ct.c_float, f32p,
                                    ct.POINTER(ct.c_int32), u32p, u32p]),
    "sv_time_step_limits": (ct.c_int, [ct.c_void_p, f32p]),
    "sv_set_frame_input": (ct.c_int, [ct.c_void_p, ct.POINTER(SvFrameInput)]),
    "sv_set_time": (ct.c_int, [ct.c_void_p, ct.c_double]),
    "sv_get_time": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_double)]),
    "sv_autotune": (ct.c_int, [ct.c_void_p, ct.c_float, f32p, ct.c_uint32, u32p, u32p]),
    "sv_set_profiling": (ct.c_int, [ct.c_void_p, ct.c_int]),
    "sv_debug_closure_wait_timeout": (ct.c_int, [ct.c_void_p, ct.c_uint64]),
    "sv_profile_report": (ct.c_int, [ct.c_void_p, ct.c_char_p, ct.c_uint64]),
    "sv_mlp_param_count": (ct.c_int, []),
    "sv_mlp_forward": (ct.c_int, [f32p, f32p, ct.c_uint64, f32p]),
    "sv_mlp_grad": (ct.c_int, [f32p, f32p, f32p, f32p, ct.c_uint64, f32p, f32p, f32p]),
    "sv_closure_harvest": (ct.c_int, [ct.c_void_p, ct.c_float, ct.c_uint32, ct.c_float, ct.c_uint32,
                                      ct.POINTER(ct.c_uint64)]),
    "sv_closure_train": (ct.c_int, [ct.c_void_p, ct.c_uint32, ct.c_uint32, ct.c_float, ct.c_uint32, f32p]),
    "sv_closure_set_mode": (ct.c_int, [ct.c_void_p, ct.c_int]),
    "sv_closure_copy": (ct.c_int, [ct.c_void_p, ct.c_void_p]),
    "sv_closure_harvest_from": (ct.c_int, [ct.c_void_p, ct.c_void_p, ct.c_float, ct.c_uint32, ct.c_float, ct.c_uint32,
                                           ct.POINTER(ct.c_uint64)]),
    "sv_closure_set_material_ranges": (ct.c_int, [ct.c_void_p, ct.c_float, ct.c_float, ct.c_float, ct.c_float]),
    "sv_closure_get_pool": (ct.c_int, [ct.c_void_p, ct.c_uint64, ct.c_uint64, f32p, f32p, f32p]),
    "sv_closure_pool": (ct.c_int, [ct.c_void_p, ct.POINTER(ct.c_uint64), ct.POINTER(ct.c_uint64)]),
    "sv_closure_phase_times": (ct.c_int, [ct.c_void_p, ct.c_float, ct.POINTER(ct.c_double)]),
    "sv_closure_evaluate": (ct.c_int, [ct.c_void_p, ct.c_float, ct.POINTER(ct.c_double)]),
    "sv_closure_get_params": (ct.c_int, [ct.c_void_p, f32p]),
}

_lib = None


def library_path() -> Path:
    return Path(os.environ.get("SQUISHY_VOLUMES_CUDA_LIB", str(_build.library_path())))


def load() -> ct.CDLL:
    """Loads libsquishy_volumes_cuda.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not path.exists():
            raise RuntimeError(
                f"{path} is missing: build the CUDA library first "
                "(python -c 'import __graft_entry__ as g; g.build()')"
            )
        lib = ct.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class SvError(RuntimeError):
    """A fatal error reported by the library (negative return code)."""


def check(rc: int) -> None:
    if rc < 0:
        msg = load().sv_last_error_string()
        raise SvError(msg.decode() if msg else f"error {rc}")


def ptr(arr, typ):
    if arr is None:
        return ct.cast(None, typ)
    return arr.ctypes.data_as(typ)
