"""ctypes binding of include/lightgraph_c.h and include/lightgraph_scene.h.

Two in-tree libraries (lightgraph_gb300/_build, made by
``lightgraph_gb300.build``) export these symbols:
  * liblightgraph_gb300.so -- the CUDA path and its C ABI (:func:`load`);
  * liblightgraph_host.so  -- host-only helpers with no CUDA code: scene
    description defaults and parsers, the EXR reader and writer, and the
    seeded synthetic scenes (:func:`load_host`).
Loading a missing library raises, so the GPU path can never silently fall back
to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LG_OK = 0
LG_ERR_INVALID = 1
LG_ERR_CUDA = 2
LG_ERR_NOMEM = 3
LG_ERR_STATE = 4
LG_ERR_TIMEOUT = 5
LG_ERR_NODEVICE = 6
LG_ERR_BUSY = 7

LG_GRID_DENSITY = 0
LG_GRID_TEMPERATURE = 1
LG_DTYPE_F32, LG_DTYPE_F16, LG_DTYPE_BF16 = 0, 1, 2
LG_LIGHT_DISTANT, LG_LIGHT_POINT, LG_LIGHT_ENV = 0, 1, 2
LG_MAX_RAMP_KEYS = 16
LG_MAX_LIGHTS = 8

LGS_VOLUME_SPHERE_FBM = 0
LGS_VOLUME_CUMULUS = 1
LGS_VOLUME_TEMPERATURE = 2

_ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of device memory", 4: "call order",
           5: "device wait timed out", 6: "no CUDA device", 7: "queue full"}


class GridDesc(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("origin", C.c_int32 * 3), ("voxel_size", C.c_double),
                ("world_origin", C.c_double * 3), ("leaf_mask", C.c_void_p)]


class ShaderC(C.Structure):
    _fields_ = [("density_scale", C.c_double), ("density_max", C.c_double),
                ("shadow_density_scale", C.c_double), ("scatter_density_scale", C.c_double),
                ("scatter_density_min", C.c_double), ("scattering", C.c_double * 3),
                ("albedo", C.c_double * 3), ("extinction", C.c_double * 3),
                ("emission_scale", C.c_double), ("scatter_scale", C.c_double),
                ("scatter_density_mask_power", C.c_double), ("ramp_n", C.c_int32), ("_pad0", C.c_int32),
                ("ramp_pos", C.c_double * LG_MAX_RAMP_KEYS), ("ramp_color", (C.c_double * 3) * LG_MAX_RAMP_KEYS),
                ("ramp_in", C.c_double), ("ramp_out", C.c_double)]


class LightC(C.Structure):
    _fields_ = [("type", C.c_int32), ("samples", C.c_int32), ("color", C.c_double * 3),
                ("intensity", C.c_double), ("dir", C.c_double * 3), ("pos", C.c_double * 3),
                ("rot", C.c_double * 9)]


class SettingsC(C.Structure):
    _fields_ = [("cutoff", C.c_double), ("step", C.c_double * 2), ("iter", C.c_int32),
                ("scatter_grid_res_factor", C.c_int32), ("pts_per_kernel", C.c_int32), ("_pad0", C.c_int32),
                ("seed", C.c_uint64)]


class CameraC(C.Structure):
    _fields_ = [("rotate", C.c_double * 3), ("translate", C.c_double * 3), ("y_rotate", C.c_double),
                ("focal", C.c_double), ("aperture", C.c_double), ("znear", C.c_double), ("zfar", C.c_double),
                ("width", C.c_int32), ("height", C.c_int32), ("samples", C.c_int32), ("_pad0", C.c_int32)]


class ScatterOptsC(C.Structure):
    _fields_ = [("scatter_count", C.c_uint32), ("target_size", C.c_uint32), ("n_estimates", C.c_uint32),
                ("hard_limit", C.c_uint32), ("growth_power", C.c_float), ("density_cutoff", C.c_float),
                ("min_dist_mult", C.c_float), ("connect_mult", C.c_float), ("seed_base", C.c_uint32),
                ("_pad0", C.c_uint32)]


class ServerOptsC(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_inflight", C.c_int32), ("queue_capacity", C.c_int32),
                ("solo_paths", C.c_int32), ("hbm_budget_bytes", C.c_uint64)]


class RequestC(C.Structure):
    _fields_ = [("volume", C.c_int32), ("n_graphs", C.c_int32), ("points", C.c_void_p), ("offsets", C.c_void_p),
                ("radius_sq", C.c_void_p), ("max_connect", C.c_int32), ("n_lights", C.c_int32),
                ("lights", C.c_void_p), ("shader", ShaderC), ("settings", SettingsC), ("camera", CameraC),
                ("point_voxel_size", C.c_double), ("env_rgb", C.c_void_p), ("env_w", C.c_int32),
                ("env_h", C.c_int32)]


P = C.c_void_p
I32, I64, U64, D, F = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_float

# name -> (restype, argtypes). Every symbol of include/lightgraph_c.h and
# include/lightgraph_scene.h is listed in one of the two tables; tests check
# that the libraries export them.
SIGNATURES = {
    "lg_create": (I32, [C.c_int, C.POINTER(P)]),
    "lg_destroy": (I32, [P]),
    "lg_last_error": (C.c_char_p, [P]),
    "lg_stream": (P, [P]),
    "lg_version": (C.c_char_p, []),
    "lg_kernel_launches": (U64, [P]),
    "lg_upload_grid": (I32, [P, C.c_int, C.POINTER(GridDesc), P, C.c_int]),
    "lg_clear_temperature": (I32, [P]),
    "lg_set_lights": (I32, [P, C.POINTER(LightC), C.c_int, P, C.c_int, C.c_int]),
    "lg_set_shader": (I32, [P, C.POINTER(ShaderC)]),
    "lg_set_settings": (I32, [P, C.POINTER(SettingsC)]),
    "lg_scatter_opts_default": (I32, [C.POINTER(ScatterOptsC)]),
    "lg_randgen_draws": (I32, [C.c_uint32, I64, P, P]),
    "lg_scatter_points": (I32, [P, C.POINTER(ScatterOptsC), C.c_int, C.c_int, P, P, P]),
    "lg_scatter_graphs": (I32, [P, C.POINTER(ScatterOptsC), C.c_int, C.c_int, C.c_int, P]),
    "lg_build_graphs": (I32, [P, C.c_int, P, P, P, C.c_int, P, P]),
    "lg_march_edges": (I32, [P, P]),
    "lg_solve_paths": (I32, [P, P]),
    "lg_vertex_light": (I32, [P, P]),
    "lg_diffuse": (I32, [P, P]),
    "lg_solve_graphs": (I32, [P, P]),
    "lg_splat": (I32, [P, D]),
    "lg_point_voxel_size": (D, [I64, P, C.c_int]),
    "lg_get_scatter_grid": (I32, [P, P, P, P]),
    "lg_get_vertex_data": (I32, [P, P, P]),
    "lg_geo_dump": (I32, [P, C.c_char_p, C.c_char_p, C.c_int]),
    "lg_render": (I32, [P, C.POINTER(CameraC), P, P, P, P]),
    "lg_render_frame": (I32, [P, C.c_int, P, P, P, C.c_int, D, C.POINTER(CameraC), P, P, P, P]),
    "lg_frame_device": (I32, [P, C.c_int, D, C.POINTER(CameraC)]),
    "lg_render_stats": (I32, [P, C.POINTER(U64), C.POINTER(U64), C.POINTER(U64)]),
    "lg_get_films": (I32, [P, P, P, P, P]),
    "lg_set_profiling": (I32, [P, C.c_int]),
    "lg_stage_times": (I32, [P, C.POINTER(D), C.c_int]),
    "lg_render_wave_times": (I32, [P, C.POINTER(D)]),  # 5 doubles
    "lg_set_graph_mode": (I32, [P, C.c_int]),
    "lg_frame_launches": (U64, [P]),
    "lg_set_fw_schedule": (I32, [P, C.c_int]),
    "lg_fw_schedule": (I32, [P, C.POINTER(C.c_int), C.POINTER(D), C.c_int]),
    "lg_fw_queue_check": (I32, [C.c_int, P, C.c_int, C.POINTER(I64)]),
    "lg_wait_timeout_check": (I32, [P, C.c_uint32]),
    "lg_fw_inner_loop_rate": (I32, [P, C.POINTER(D), P]),
    "lg_expm1_check": (I32, [P, P, P, P, I32]),
    "lg_fw_device": (I32, [P, C.c_int, C.c_int, P]),
    "lg_fw_host": (I32, [P, P, C.c_int]),
    "lg_diffuse_noalloc": (I32, [P, C.c_int, C.c_int, P, P, C.POINTER(D), P]),
    "lg_server_create": (I32, [C.POINTER(ServerOptsC), C.POINTER(P)]),
    "lg_server_destroy": (I32, [P]),
    "lg_server_last_error": (C.c_char_p, [P]),
    "lg_server_add_volume": (I32, [P, C.POINTER(GridDesc), P, C.POINTER(GridDesc), P, C.c_int,
                                   C.POINTER(C.c_int32)]),
    "lg_server_submit": (I32, [P, C.POINTER(RequestC), C.POINTER(I64)]),
    "lg_server_poll": (I32, [P, I64, C.POINTER(C.c_int)]),
    "lg_server_wait": (I32, [P, I64, C.c_int, P, C.POINTER(D), C.POINTER(D)]),
    "lg_request_bytes": (U64, [C.POINTER(RequestC)]),
    "lg_server_stats": (I32, [P, C.POINTER(U64), C.POINTER(U64)]),
}

# liblightgraph_host.so: scene description helpers, EXR files, synthetic scenes
HOST_SIGNATURES = {
    "lg_read_exr_rgba": (I32, [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), P]),
    "lg_write_exr": (I32, [C.c_char_p, C.c_int, C.c_int, C.c_int, P, P]),
    "lg_shader_default": (None, [C.POINTER(ShaderC)]),
    "lg_shader_set_coefficients": (None, [C.POINTER(ShaderC), C.POINTER(D), C.POINTER(D), C.POINTER(D)]),
    "lg_settings_default": (None, [C.POINTER(SettingsC)]),
    "lg_camera_default": (None, [C.POINTER(CameraC)]),
    "lg_parse_light": (I32, [C.c_char_p, C.POINTER(LightC)]),
    "lg_parse_color_ramp": (I32, [C.c_char_p, C.POINTER(ShaderC)]),
    "lgs_volume": (I64, [C.c_int, C.c_int, C.c_int, U64, D, P, P]),
    "lgs_points": (I64, [P, C.c_int, D, I64, U64, D, I64, P]),
    "lgs_envmap": (None, [C.c_int, C.c_int, D, D, D, D, P]),
}

_lib = None
_host = None


def _open(path: str, table: dict) -> C.CDLL:
    if not os.path.exists(path):
        raise ImportError(
            f"lightgraph_gb300 native library missing at {path}; run "
            "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc for sm_103a)")
    lib = C.CDLL(path)
    for name, (res, args) in table.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load() -> C.CDLL:
    """Load the in-tree CUDA library; raise if it has not been built."""
    global _lib
    if _lib is None:
        _lib = _open(_build.lib_path(), SIGNATURES)
    return _lib


def load_host() -> C.CDLL:
    """Load the in-tree host-only helper library; raise if it has not been built."""
    global _host
    if _host is None:
        _host = _open(_build.host_lib_path(), HOST_SIGNATURES)
    return _host


class LightGraphError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{_ERRORS.get(status, 'error')} ({status}): {msg}")
        self.status = status


def ptr(a) -> int | None:
    """Data pointer of a numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data
