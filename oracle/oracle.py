"""TEST INFRASTRUCTURE ONLY: ctypes driver of the C restatement in
rast_oracle.c (the CPU oracle the CUDA kernels are checked against).

Parity against the reference's JAX execution is unpinned (JAX is not
installable here); the restatement is checked against the reference's own
smoke-test assertions in tests/.  Only tests, the smoke check and the CPU
baseline of bench.py use this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from ctypes import POINTER, c_double, c_float, c_int, c_longlong, c_void_p
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SRC = HERE / "rast_oracle.c"
HDR = HERE / "rast_oracle.h"

CFLAGS = ["-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-std=c11"]


def _lib_path(double: bool) -> Path:
    return BUILD / ("liboracle_f64.so" if double else "liboracle_f32.so")


def build(force: bool = False) -> None:
    """Compile the oracle (float and double builds) with gcc."""
    BUILD.mkdir(parents=True, exist_ok=True)
    for double in (False, True):
        out = _lib_path(double)
        if not force and out.exists() and out.stat().st_mtime >= max(SRC.stat().st_mtime, HDR.stat().st_mtime):
            continue
        tmp = out.with_suffix(".tmp")
        cmd = [os.environ.get("CC", "gcc"), *CFLAGS, f"-DOR_DOUBLE={int(double)}", "-o", str(tmp), str(SRC), "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, out)


def _scene_struct(real):
    R = POINTER(real)
    I = POINTER(c_int)
    R3 = real * 3

    class Scene(ctypes.Structure):
        _fields_ = [
            ("shader", c_int), ("width", c_int), ("height", c_int), ("n_threads", c_int),
            ("viewport", R), ("world_to_clip", R), ("world_to_eye_norm", R),
            ("n_verts", c_int), ("position", R), ("normal", R), ("uv", R), ("colour", R),
            ("texture_index", I), ("id_to_face", I), ("darboux_faces", I), ("n_darboux_faces", c_int),
            ("n_faces", c_int), ("faces", I),
            ("light_direction", R3), ("light_colour", R3), ("light_dir_eye", R3),
            ("ambient", R3), ("diffuse", R3), ("specular", R3),
            ("texture", R), ("tex_w", c_int), ("tex_h", c_int), ("tex_c", c_int),
            ("specular_map", R), ("spec_w", c_int), ("spec_h", c_int),
            ("normal_map", R), ("nm_w", c_int), ("nm_h", c_int),
            ("texture_shape", I), ("n_objects", c_int), ("texture_offset", c_int),
            ("shadow_map", R), ("shadow_w", c_int), ("shadow_h", c_int),
            ("shadow_world_to_clip", R), ("shadow_viewport", R), ("shadow_strength", R3),
            ("zbuffer", R), ("canvas", R), ("prim_id", I), ("near_ties", c_longlong),
            ("layers", c_int), ("mixer", c_int), ("opacity", real), ("background", R3), ("face_alpha", R),
            ("x_begin", c_int), ("x_end", c_int), ("y_begin", c_int), ("y_end", c_int), ("branch", I),
            ("texel", I),
        ]

    return Scene


SceneF32 = _scene_struct(c_float)
SceneF64 = _scene_struct(c_double)
_LIBS = {}


def _load(double: bool):
    if double not in _LIBS:
        build()
        lib = ctypes.CDLL(str(_lib_path(double)))
        fn = lib.or_render_f64 if double else lib.or_render_f32
        fn.restype = c_int
        fn.argtypes = [c_void_p]
        if not double:
            lib.or_inv3_f32.argtypes = [POINTER(c_float), POINTER(c_float)]
            lib.or_det3_f32.restype = c_float
            lib.or_det3_f32.argtypes = [POINTER(c_float)]
            lib.or_depth_order_f32.restype = ctypes.c_uint
            lib.or_depth_order_f32.argtypes = [c_float]
        _LIBS[double] = lib
    return _LIBS[double]


def _np(x, dtype):
    if x is None:
        return None
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(x), dtype=dtype)


def render(spec, zbuffer, canvas=None, n_threads: int = 1, dtype=np.float32, window=None,
           want_branch: bool = False):
    """Render one job described by `spec` (attributes as jaxrenderer_gb300's
    JobSpec) on the CPU.  Returns dict(zbuffer, canvas, prim_id, near_ties),
    plus `branch` (the per-pixel branch signature) and `texel` (the diffuse
    texel row sampled, -1 where none) with `want_branch` (rast_oracle.h).  `window` = (x0, x1, y0, y1) renders only those pixels;
    the others keep their input values (prim_id -1, branch 0)."""
    double = np.dtype(dtype) == np.float64
    real = c_double if double else c_float
    Scene = SceneF64 if double else SceneF32
    lib = _load(double)
    keep = []

    def rp(x):
        a = _np(x, dtype)
        if a is None:
            return None
        keep.append(a)
        return a.ctypes.data_as(POINTER(real))

    def ip(x):
        a = _np(x, np.int32)
        if a is None:
            return None
        keep.append(a)
        return a.ctypes.data_as(POINTER(c_int))

    s = Scene()
    s.shader = int(spec.shader)
    s.width, s.height = int(spec.width), int(spec.height)
    s.n_threads = int(n_threads)
    s.viewport, s.world_to_clip, s.world_to_eye_norm = rp(spec.viewport), rp(spec.world_to_clip), rp(spec.world_to_eye_norm)
    pos = _np(spec.position, dtype)
    s.n_verts = int(pos.shape[0])
    s.position = rp(pos)
    s.normal, s.uv, s.colour = rp(spec.normal), rp(spec.uv), rp(spec.colour)
    s.texture_index, s.id_to_face = ip(spec.texture_index), ip(spec.id_to_face)
    if spec.darboux_faces is not None:
        s.darboux_faces = ip(spec.darboux_faces)
        s.n_darboux_faces = int(np.asarray(_np(spec.darboux_faces, np.int32)).shape[0])
    faces = _np(spec.faces, np.int32).reshape(-1, 3)
    s.n_faces = int(faces.shape[0])
    s.faces = ip(faces)
    for name in ("light_direction", "light_colour", "light_dir_eye", "ambient", "diffuse", "specular", "shadow_strength"):
        v = _np(getattr(spec, name), dtype).reshape(-1)
        if v.size == 1:
            v = np.repeat(v, 3)
        arr = getattr(s, name)
        for k in range(3):
            arr[k] = float(v[k])
    if spec.texture is not None:
        t = _np(spec.texture, dtype)
        if t.ndim == 2:
            t = t[..., None]
        s.texture = rp(t)
        s.tex_w, s.tex_h, s.tex_c = t.shape[:3]
    if spec.specular_map is not None:
        sm = _np(spec.specular_map, dtype)
        s.specular_map = rp(sm)
        s.spec_w, s.spec_h = sm.shape[:2]
    if spec.normal_map is not None:
        nm = _np(spec.normal_map, dtype)
        s.normal_map = rp(nm)
        s.nm_w, s.nm_h = nm.shape[:2]
    if spec.texture_shape is not None:
        ts = _np(spec.texture_shape, np.int32).reshape(-1, 2)
        s.texture_shape = ip(ts)
        s.n_objects = ts.shape[0]
    s.texture_offset = int(spec.texture_offset)
    if spec.shadow_map is not None:
        shm = _np(spec.shadow_map, dtype)
        s.shadow_map = rp(shm)
        s.shadow_w, s.shadow_h = shm.shape[:2]
    s.shadow_world_to_clip = rp(spec.shadow_world_to_clip)
    s.shadow_viewport = rp(spec.shadow_viewport)
    s.layers = int(getattr(spec, "layers", 0))
    s.mixer = int(getattr(spec, "mixer", 0))
    s.opacity = float(getattr(spec, "opacity", 1.0))
    bg = _np(getattr(spec, "background", (0.0, 0.0, 0.0)), dtype).reshape(-1)
    if bg.size == 1:
        bg = np.repeat(bg, 3)
    for k in range(3):
        s.background[k] = float(bg[k])
    if getattr(spec, "face_alpha", None) is not None:
        s.face_alpha = rp(_np(spec.face_alpha, dtype).reshape(-1))
    z = np.array(_np(zbuffer, dtype), copy=True)
    s.zbuffer = z.ctypes.data_as(POINTER(real))
    c = None
    if canvas is not None:
        c = np.array(_np(canvas, dtype), copy=True)
        s.canvas = c.ctypes.data_as(POINTER(real))
    pid = np.full((s.width, s.height), -1, dtype=np.int32)
    s.prim_id = pid.ctypes.data_as(POINTER(c_int))
    if window is not None:
        x0, x1, y0, y1 = (int(v) for v in window)
        if x1 <= x0 or y1 <= y0:
            raise ValueError(f"empty window {window}")
        s.x_begin, s.x_end, s.y_begin, s.y_end = x0, x1, y0, y1
    branch = texel = None
    if want_branch:
        branch = np.zeros((s.width, s.height), dtype=np.int32)
        s.branch = branch.ctypes.data_as(POINTER(c_int))
        texel = np.full((s.width, s.height), -1, dtype=np.int32)
        s.texel = texel.ctypes.data_as(POINTER(c_int))
    st = lib.or_render_f64(ctypes.byref(s)) if double else lib.or_render_f32(ctypes.byref(s))
    if st != 0:
        raise RuntimeError(f"oracle render failed: {st}")
    if getattr(spec, "apply_depth_offset", False):
        z = (z + np.asarray(spec.depth_offset, dtype=dtype)).astype(dtype)
    out = {"zbuffer": z, "canvas": c, "prim_id": pid, "near_ties": int(s.near_ties)}
    if branch is not None:
        out["branch"] = branch
        out["texel"] = texel
    return out


def inv3(m) -> np.ndarray:
    lib = _load(False)
    a = np.ascontiguousarray(np.asarray(m, np.float32).reshape(9))
    out = np.zeros(9, np.float32)
    lib.or_inv3_f32(a.ctypes.data_as(POINTER(c_float)), out.ctypes.data_as(POINTER(c_float)))
    return out.reshape(3, 3)


def det3(m) -> np.float32:
    lib = _load(False)
    a = np.ascontiguousarray(np.asarray(m, np.float32).reshape(9))
    return np.float32(lib.or_det3_f32(a.ctypes.data_as(POINTER(c_float))))


def depth_order(z: float) -> int:
    return int(_load(False).or_depth_order_f32(float(np.float32(z))))
