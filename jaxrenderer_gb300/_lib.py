"""ctypes binding of `include/rast_gb300.h` (the C ABI of librast_gb300.so).

The structures below mirror the header field by field; `tests/` checks the
offsets against a C compiler's.  Loading fails loudly when the library has
not been built: there is no CPU fallback for the rasterisation path.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_float, c_int, c_int32, c_int64, c_size_t, c_uint64, c_void_p
from pathlib import Path

from . import _build

SHADER_DEPTH = 0
SHADER_GOURAUD = 1
SHADER_GOURAUD_TEXTURE = 2
SHADER_PHONG = 3
SHADER_PHONG_DARBOUX = 4
SHADER_PHONG_REFLECTION = 5
SHADER_PHONG_REFLECTION_SHADOW = 6

ABI_VERSION = 6  # RAST_ABI_VERSION of the header these structures mirror

JOB_APPLY_DEPTH_OFFSET = 1
JOB_FACE_ALPHA = 2

MAX_LAYERS = 4
MIX_NEAREST = 0
MIX_OVER = 1

STATUS_NAMES = {
    0: "RAST_OK",
    1: "RAST_ERR_INVALID_ARGUMENT",
    2: "RAST_ERR_WORKSPACE_TOO_SMALL",
    3: "RAST_ERR_CUDA",
    4: "RAST_ERR_UNSUPPORTED",
    5: "RAST_ERR_TIMEOUT",
    6: "RAST_ERR_BIN_OVERFLOW",
    7: "RAST_ERR_INDEX_OUT_OF_RANGE",
    8: "RAST_ERR_STATIC_SCRATCH_TOO_SMALL",
}
STATIC_SCRATCH_BYTES = 64 << 20
PHASE_COVERAGE = 1
PHASE_SHADE = 2

F16 = c_float * 16
F3 = c_float * 3


class RastJob(ctypes.Structure):
    _fields_ = [
        ("shader", c_int32),
        ("width", c_int32),
        ("height", c_int32),
        ("n_verts", c_int32),
        ("n_faces", c_int32),
        ("n_darboux_faces", c_int32),
        ("n_objects", c_int32),
        ("texture_offset", c_int32),
        ("vert_begin", c_int64),
        ("face_begin", c_int64),
        ("darboux_face_begin", c_int64),
        ("pixel_begin", c_int64),
        ("vout_begin", c_int64),
        ("setup_begin", c_int64),
        ("texture_begin", c_int64),
        ("specular_begin", c_int64),
        ("normal_map_begin", c_int64),
        ("texture_shape_begin", c_int64),
        ("shadow_begin", c_int64),
        ("tex_w", c_int32),
        ("tex_h", c_int32),
        ("tex_c", c_int32),
        ("spec_w", c_int32),
        ("spec_h", c_int32),
        ("nm_w", c_int32),
        ("nm_h", c_int32),
        ("shadow_w", c_int32),
        ("shadow_h", c_int32),
        ("depth_offset", c_float),
        ("viewport", F16),
        ("world_to_clip", F16),
        ("world_to_eye_norm", F16),
        ("shadow_viewport", F16),
        ("shadow_world_to_clip", F16),
        ("light_direction", F3),
        ("light_colour", F3),
        ("light_dir_eye", F3),
        ("ambient", F3),
        ("diffuse", F3),
        ("specular", F3),
        ("shadow_strength", F3),
        ("flags", c_int32),
        ("layers", c_int32),
        ("mixer", c_int32),
        ("opacity", c_float),
        ("background", F3),
        ("reserved", c_int32),
    ]


class RastPools(ctypes.Structure):
    _fields_ = [
        ("position", c_void_p),
        ("normal", c_void_p),
        ("uv", c_void_p),
        ("colour", c_void_p),
        ("texture_index", c_void_p),
        ("id_to_face", c_void_p),
        ("faces", c_void_p),
        ("darboux_faces", c_void_p),
        ("texture", c_void_p),
        ("specular_map", c_void_p),
        ("normal_map", c_void_p),
        ("texture_shape", c_void_p),
        ("shadow_map", c_void_p),
        ("zbuffer", c_void_p),
        ("canvas", c_void_p),
        ("prim_id", c_void_p),
        ("face_alpha", c_void_p),
        ("layer_prim", c_void_p),
    ]


class RastBatch(ctypes.Structure):
    _fields_ = [
        ("jobs", c_void_p),
        ("n_jobs", c_int32),
        ("max_width", c_int32),
        ("max_height", c_int32),
        ("max_verts", c_int32),
        ("max_faces", c_int32),
        ("shader_mask", c_int32),
        ("total_vout", c_int64),
        ("total_setup", c_int64),
        ("total_pixels", c_int64),
        ("pools", RastPools),
        ("near_ties", c_void_p),
        ("max_layers", c_int32),
        ("reserved", c_int32),
    ]


class RastProfile(ctypes.Structure):
    _fields_ = [("n", c_int32), ("ms", c_float * 16), ("names", ctypes.c_char_p * 16)]


class RastTiledConfig(ctypes.Structure):
    _fields_ = [("tile_w", c_int32), ("tile_h", c_int32), ("bin_capacity", c_uint64), ("small_area", c_int32),
                ("warps_per_tile", c_int32)]


class RastTiledStats(ctypes.Structure):
    _fields_ = [("bin_entries", c_uint64), ("bin_capacity", c_uint64), ("tiles", c_uint64),
                ("overflow", ctypes.c_uint32), ("binned_faces", ctypes.c_uint32), ("pixel_tests", c_uint64)]


GRAD_WORLD_TO_CLIP = 0
GRAD_WORLD_TO_EYE_NORM = 16
GRAD_LIGHT_DIRECTION = 32
GRAD_LIGHT_COLOUR = 35
GRAD_LIGHT_DIR_EYE = 38
GRAD_AMBIENT = 41
GRAD_DIFFUSE = 44
GRAD_SPECULAR = 47
GRAD_SHADOW_STRENGTH = 50
GRAD_BACKGROUND = 53
NPARAM = 56


class RastGradPools(ctypes.Structure):
    _fields_ = [("position", c_void_p), ("normal", c_void_p), ("colour", c_void_p), ("texture", c_void_p),
                ("specular_map", c_void_p), ("job_params", c_void_p), ("normal_map", c_void_p)]


# Exported symbols and their prototypes: (name, restype, argtypes).
class RastMesh(ctypes.Structure):
    _fields_ = [("vert_begin", c_int64), ("norm_begin", c_int64), ("uv_begin", c_int64), ("face_begin", c_int64),
                ("n_verts", c_int32), ("n_norms", c_int32), ("n_uvs", c_int32), ("n_faces", c_int32)]


class RastInstance(ctypes.Structure):
    _fields_ = [("mesh", c_int32), ("scene_first", c_int32), ("scene_count", c_int32),
                ("vert_offset", c_int32), ("norm_offset", c_int32), ("uv_offset", c_int32),
                ("scene_verts", c_int32), ("scene_norms", c_int32), ("scene_uvs", c_int32),
                ("reserved", c_int32), ("corner_begin", c_int64), ("vert_row", c_int64), ("norm_row", c_int64),
                ("uv_row", c_int64)]


class RastMergeBatch(ctypes.Structure):
    _fields_ = [("meshes", c_void_p), ("n_meshes", c_int32), ("n_instances", c_int32), ("instances", c_void_p),
                ("transforms", c_void_p), ("local_scaling", c_void_p), ("mesh_verts", c_void_p),
                ("mesh_norms", c_void_p), ("mesh_uvs", c_void_p), ("mesh_faces", c_void_p),
                ("mesh_faces_norm", c_void_p), ("mesh_faces_uv", c_void_p), ("total_faces", c_int64),
                ("total_verts", c_int64), ("total_norms", c_int64), ("total_uvs", c_int64),
                ("position", c_void_p), ("normal", c_void_p),
                ("uv", c_void_p), ("texture_index", c_void_p)]


PROTOTYPES = [
    ("rast_plain_workspace_bytes", c_size_t, [POINTER(RastBatch)]),
    ("rast_render_plain", c_int, [POINTER(RastBatch), c_void_p, c_size_t, c_void_p]),
    ("rast_render_plain_profiled", c_int, [POINTER(RastBatch), c_void_p, c_size_t, c_void_p, POINTER(RastProfile)]),
    ("rast_tiled_workspace_bytes", c_size_t, [POINTER(RastBatch), POINTER(RastTiledConfig)]),
    ("rast_render_tiled", c_int, [POINTER(RastBatch), POINTER(RastTiledConfig), c_void_p, c_size_t, c_void_p]),
    ("rast_render_tiled_profiled", c_int,
     [POINTER(RastBatch), POINTER(RastTiledConfig), c_void_p, c_size_t, c_void_p, POINTER(RastProfile)]),
    ("rast_render_tiled_static", c_int, [POINTER(RastBatch), POINTER(RastTiledConfig), c_void_p]),
    ("rast_autotune", c_int, [POINTER(RastBatch), c_void_p, POINTER(RastTiledConfig)]),
    ("rast_render_tiled_phase", c_int, [POINTER(RastBatch), POINTER(RastTiledConfig), c_void_p, c_size_t, c_void_p,
                                        c_int]),
    ("rast_tiled_stats", c_int,
     [POINTER(RastBatch), POINTER(RastTiledConfig), c_void_p, c_void_p, POINTER(RastTiledStats)]),
    ("rast_backward_workspace_bytes", c_size_t, [POINTER(RastBatch)]),
    ("rast_backward", c_int,
     [POINTER(RastBatch), c_void_p, c_void_p, POINTER(RastGradPools), c_void_p, c_size_t, c_void_p]),
    ("rast_backward_profiled", c_int,
     [POINTER(RastBatch), c_void_p, c_void_p, POINTER(RastGradPools), c_void_p, c_size_t, c_void_p,
      POINTER(RastProfile)]),
    ("rast_backward_mse", c_int,
     [POINTER(RastBatch), c_void_p, ctypes.c_float, c_void_p, POINTER(RastGradPools), c_void_p, c_size_t, c_void_p]),
    ("rast_merge_workspace_bytes", c_size_t, [POINTER(RastMergeBatch)]),
    ("rast_merge_objects", c_int, [POINTER(RastMergeBatch), c_void_p, c_size_t, c_void_p]),
    ("rast_display_u8", c_int, [c_void_p, c_int64, c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p]),
    ("rast_validate_job", c_int, [POINTER(RastJob)]),
    ("rast_error_string", ctypes.c_char_p, [c_int]),
    ("rast_abi_version", c_int, []),
]

_LIB = None


class RastError(RuntimeError):
    """A non-zero RastStatus returned by the CUDA library."""

    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}")


def library_path() -> Path:
    return _build.library_path()


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load librast_gb300.so (building it first when it is missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists() or not _build.up_to_date():
        if not build_if_missing:
            raise RuntimeError(f"{path} is not built; run jaxrenderer_gb300._build.build()")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, res, args in PROTOTYPES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.rast_abi_version() != ABI_VERSION:
        raise RuntimeError("librast_gb300.so ABI version mismatch")
    _LIB = lib
    return lib


def check(status: int, where: str) -> None:
    if status != 0:
        raise RastError(status, where)


def as_c_floats(dst, values) -> None:
    for k, v in enumerate(values):
        dst[k] = float(v)


__all__ = [
    "RastJob",
    "RastPools",
    "RastBatch",
    "RastProfile",
    "RastTiledConfig",
    "RastTiledStats",
    "RastGradPools",
    "RastError",
    "PROTOTYPES",
    "load",
    "check",
    "c_uint64",
]
