"""Host side of the C ABI: one `JobSpec` per pipeline.render call, packed
into a `RastBatch` (pools of flat device arrays + a device array of RastJob)
and rendered by librast_gb300.so.

`JobSpec` holds host (NumPy) or device (torch) arrays exactly as the
reference's `*ExtraInput` NamedTuples hand them to pipeline.render; the
per-shader extraction is `job_from_extra`.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Any, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from .geometry import Camera, _arr

F32 = np.float32
I32 = np.int32

_TEXTURED = {
    _lib.SHADER_GOURAUD_TEXTURE,
    _lib.SHADER_PHONG,
    _lib.SHADER_PHONG_DARBOUX,
    _lib.SHADER_PHONG_REFLECTION,
    _lib.SHADER_PHONG_REFLECTION_SHADOW,
}
_REFLECTION = {_lib.SHADER_PHONG_REFLECTION, _lib.SHADER_PHONG_REFLECTION_SHADOW}


@dataclass
class JobSpec:
    """Inputs of one pipeline.render call (shader + camera + extra + size)."""

    shader: int
    width: int
    height: int
    viewport: np.ndarray
    world_to_clip: np.ndarray
    world_to_eye_norm: np.ndarray
    position: Any
    faces: Any
    normal: Any = None
    uv: Any = None
    colour: Any = None
    texture_index: Any = None
    id_to_face: Any = None
    darboux_faces: Any = None
    light_direction: np.ndarray = field(default_factory=lambda: np.array((0.0, 0.0, -1.0), F32))
    light_colour: np.ndarray = field(default_factory=lambda: np.ones(3, F32))
    light_dir_eye: np.ndarray = field(default_factory=lambda: np.zeros(3, F32))
    ambient: np.ndarray = field(default_factory=lambda: np.zeros(3, F32))
    diffuse: np.ndarray = field(default_factory=lambda: np.zeros(3, F32))
    specular: np.ndarray = field(default_factory=lambda: np.zeros(3, F32))
    texture: Any = None
    specular_map: Any = None
    normal_map: Any = None
    texture_shape: Any = None
    texture_offset: int = 0
    shadow_map: Any = None
    shadow_viewport: np.ndarray = field(default_factory=lambda: np.identity(4, dtype=F32))
    shadow_world_to_clip: np.ndarray = field(default_factory=lambda: np.identity(4, dtype=F32))
    shadow_strength: np.ndarray = field(default_factory=lambda: np.zeros(3, F32))
    depth_offset: float = 0.0
    apply_depth_offset: bool = False
    # compiled primitive_chooser / mix hooks (rast_gb300.h, RastMixer):
    # layers 0 = the default chooser, 1..4 = that many nearest candidates
    layers: int = 0
    mixer: int = 0  # _lib.MIX_NEAREST or _lib.MIX_OVER
    opacity: float = 1.0  # MIX_OVER, every face (without face_alpha)
    background: Any = (0.0, 0.0, 0.0)  # MIX_OVER, seen through the last layer
    face_alpha: Any = None  # MIX_OVER, (F,) opacity per face

    @property
    def n_verts(self) -> int:
        return int(self.position.shape[0])

    @property
    def n_faces(self) -> int:
        return int(self.faces.shape[0])


def _f3(x) -> np.ndarray:
    a = _arr(x, F32).reshape(-1)
    if a.size == 1:
        a = np.repeat(a, 3)
    return a[:3].astype(F32)


def _host_or_device(x, dtype):
    if isinstance(x, torch.Tensor):
        return x
    return np.ascontiguousarray(np.asarray(x), dtype=dtype)


def job_from_extra(shader_id: int, camera: Camera, extra, width: int, height: int) -> JobSpec:
    """Map a shader's ExtraInput NamedTuple onto a JobSpec.

    Field names follow the reference's ExtraInput classes
    (renderer/shaders/*.py)."""
    spec = JobSpec(
        shader=shader_id,
        width=int(width),
        height=int(height),
        viewport=_arr(camera.viewport, F32),
        world_to_clip=_arr(camera.world_to_clip, F32),
        world_to_eye_norm=_arr(camera.world_to_eye_norm, F32),
        position=_host_or_device(extra.position, F32),
        faces=None,
    )
    if shader_id != _lib.SHADER_DEPTH:
        light = extra.light
        spec.light_direction = _f3(light.direction)
        spec.light_colour = _f3(light.colour)
        spec.normal = _host_or_device(extra.normal, F32)
    if shader_id == _lib.SHADER_GOURAUD:
        spec.colour = _host_or_device(extra.colour, F32)
    if shader_id in _TEXTURED:
        spec.uv = _host_or_device(extra.uv, F32)
        tex = _host_or_device(extra.texture, F32)
        if tex.ndim == 2:
            tex = tex[..., None] if isinstance(tex, np.ndarray) else tex.unsqueeze(-1)
        spec.texture = tex
    if shader_id == _lib.SHADER_PHONG_DARBOUX:
        spec.normal_map = _host_or_device(extra.normal_map, F32)
        spec.id_to_face = _host_or_device(extra.id_to_face, I32)
        spec.darboux_faces = _host_or_device(extra.faces_indices, I32)
    if shader_id in _REFLECTION:
        spec.light_dir_eye = _f3(extra.light_dir_eye)
        spec.texture_shape = _host_or_device(extra.texture_shape, I32).reshape(-1, 2)
        spec.texture_index = _host_or_device(extra.texture_index, I32)
        spec.texture_offset = int(np.asarray(extra.texture_offset))
        spec.specular_map = _host_or_device(extra.specular_map, F32)
        spec.ambient = _f3(extra.ambient)
        spec.diffuse = _f3(extra.diffuse)
        spec.specular = _f3(extra.specular)
    if shader_id == _lib.SHADER_PHONG_REFLECTION_SHADOW:
        shadow = extra.shadow
        spec.shadow_map = shadow.shadow_map
        spec.shadow_viewport = _arr(shadow.camera.viewport, F32)
        spec.shadow_world_to_clip = _arr(shadow.camera.world_to_clip, F32)
        spec.shadow_strength = _f3(shadow.strength)
    return spec


# ---------------------------------------------------------------- packing


def _to_dev(x, dtype: torch.dtype, device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(x)).to(device=device, dtype=dtype)


class _Pool:
    """Concatenation of per-job arrays into one flat device array."""

    def __init__(self, dtype: torch.dtype, row: int):
        self.dtype = dtype
        self.row = row  # elements per row
        self.parts: List[Any] = []
        self.rows = 0

    def add(self, x) -> int:
        """Append x; returns its first row (or 0 when x is None)."""
        if x is None:
            return 0
        begin = self.rows
        n = int(np.prod(tuple(x.shape))) // self.row
        self.parts.append(x)
        self.rows += n
        return begin

    def tensor(self, device) -> Optional[torch.Tensor]:
        if not self.parts:
            return None
        ts = [_to_dev(p, self.dtype, device).reshape(-1) for p in self.parts]
        return ts[0] if len(ts) == 1 else torch.cat(ts)


def _ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    return None if t is None else t.data_ptr()


@dataclass
class PackedBatch:
    batch: _lib.RastBatch
    keep: list  # tensors that must outlive the call
    zbuffer: torch.Tensor
    canvas: Optional[torch.Tensor]
    prim_id: Optional[torch.Tensor]
    near_ties: Optional[torch.Tensor]
    pixel_begin: List[int]
    pools: dict = None  # name -> device tensor (RastPools inputs)
    jobs: object = None  # ctypes array of RastJob (host copy)
    layer_prim: Optional[torch.Tensor] = None  # (MAX_LAYERS, pixels) slots of layered jobs


def pack(specs: Sequence[JobSpec], zbuffers: Sequence[Any], canvases: Sequence[Any], device,
         want_prim_id: bool = True, count_ties: bool = False) -> PackedBatch:
    """Pack jobs + their initial buffers into a RastBatch."""
    n = len(specs)
    if n < 1 or n > 65535:
        raise ValueError("a batch holds 1..65535 jobs")
    jobs = (_lib.RastJob * n)()
    pos, nrm, uvp, col = _Pool(torch.float32, 3), _Pool(torch.float32, 3), _Pool(torch.float32, 2), _Pool(torch.float32, 3)
    tix, i2f = _Pool(torch.int32, 1), _Pool(torch.int32, 1)
    fac, dfc = _Pool(torch.int32, 3), _Pool(torch.int32, 3)
    tex, spm, nmp, tsh, shm = (_Pool(torch.float32, 1), _Pool(torch.float32, 1), _Pool(torch.float32, 1),
                               _Pool(torch.int32, 2), _Pool(torch.float32, 1))
    zb, cv = _Pool(torch.float32, 1), _Pool(torch.float32, 3)
    alp = _Pool(torch.float32, 1)  # row-aligned with faces
    max_layers = 0
    vout = setup = pixels = 0
    pixel_begin = []
    mask = 0
    maxw = maxh = maxv = maxf = 0
    for k, s in enumerate(specs):
        J = jobs[k]
        V, F = s.n_verts, (0 if s.faces is None else s.n_faces)
        J.shader = s.shader
        J.width, J.height = s.width, s.height
        J.n_verts, J.n_faces = V, F
        J.vert_begin = pos.add(s.position)
        # every vertex pool stays row-aligned with position
        for pool, arr in ((nrm, s.normal), (uvp, s.uv), (col, s.colour), (tix, s.texture_index), (i2f, s.id_to_face)):
            if arr is not None:
                if pool.rows < J.vert_begin:
                    pool.add(np.zeros((J.vert_begin - pool.rows, pool.row), np.float32 if pool.dtype == torch.float32 else np.int32))
                pool.add(arr)
        J.face_begin = fac.add(s.faces)
        if s.face_alpha is not None:
            fa = _host_or_device(s.face_alpha, np.float32).reshape(-1)
            if int(fa.shape[0]) != F:
                raise ValueError(f"job {k}: face_alpha has {int(fa.shape[0])} entries for {F} faces")
            if alp.rows < J.face_begin:
                alp.add(np.zeros(J.face_begin - alp.rows, np.float32))
            alp.add(fa)
        if s.darboux_faces is not None:
            J.darboux_face_begin = dfc.add(s.darboux_faces)
            J.n_darboux_faces = int(s.darboux_faces.shape[0])
        J.pixel_begin = pixels
        pixel_begin.append(pixels)
        J.vout_begin = vout
        J.setup_begin = setup
        vout += V
        setup += F
        pixels += s.width * s.height
        if s.texture is not None:
            J.texture_begin = tex.add(s.texture)
            J.tex_w, J.tex_h, J.tex_c = (int(d) for d in s.texture.shape[:3])
        if s.specular_map is not None:
            J.specular_begin = spm.add(s.specular_map)
            J.spec_w, J.spec_h = (int(d) for d in s.specular_map.shape[:2])
        if s.normal_map is not None:
            J.normal_map_begin = nmp.add(s.normal_map)
            J.nm_w, J.nm_h = (int(d) for d in s.normal_map.shape[:2])
        if s.texture_shape is not None:
            J.texture_shape_begin = tsh.add(s.texture_shape)
            J.n_objects = int(s.texture_shape.shape[0])
        J.texture_offset = int(s.texture_offset)
        if s.shadow_map is not None:
            J.shadow_begin = shm.add(s.shadow_map)
            J.shadow_w, J.shadow_h = (int(d) for d in s.shadow_map.shape[:2])
        J.depth_offset = float(np.float32(s.depth_offset))
        J.flags = (_lib.JOB_APPLY_DEPTH_OFFSET if s.apply_depth_offset else 0) | (
            _lib.JOB_FACE_ALPHA if s.face_alpha is not None else 0)
        J.layers, J.mixer = int(s.layers), int(s.mixer)
        J.opacity = float(np.float32(s.opacity))
        _lib.as_c_floats(J.background, _f3(s.background))
        max_layers = max(max_layers, J.layers)
        for name in ("viewport", "world_to_clip", "world_to_eye_norm", "shadow_viewport", "shadow_world_to_clip"):
            _lib.as_c_floats(getattr(J, name), np.asarray(getattr(s, name), F32).reshape(-1))
        for name in ("light_direction", "light_colour", "light_dir_eye", "ambient", "diffuse", "specular", "shadow_strength"):
            _lib.as_c_floats(getattr(J, name), _f3(getattr(s, name)))
        st = _lib.load().rast_validate_job(ctypes.byref(J))
        _lib.check(st, f"job {k}")
        zb.add(zbuffers[k])
        if canvases[k] is not None:
            if cv.rows < J.pixel_begin:
                cv.add(np.zeros((J.pixel_begin - cv.rows, 3), np.float32))
            cv.add(canvases[k])
        mask |= 1 << s.shader
        maxw, maxh, maxv, maxf = max(maxw, s.width), max(maxh, s.height), max(maxv, V), max(maxf, F)

    keep = []

    def dev(pool):
        t = pool.tensor(device)
        if t is not None:
            keep.append(t)
        return t

    tensors = {name: dev(p) for name, p in (
        ("position", pos), ("normal", nrm), ("uv", uvp), ("colour", col), ("texture_index", tix),
        ("id_to_face", i2f), ("faces", fac), ("darboux_faces", dfc), ("texture", tex),
        ("specular_map", spm), ("normal_map", nmp), ("texture_shape", tsh), ("shadow_map", shm),
        ("face_alpha", alp))}
    zbuf = zb.tensor(device).clone()
    canvas = None
    if cv.parts:
        if cv.rows < pixels:
            cv.add(np.zeros((pixels - cv.rows, 3), np.float32))
        canvas = cv.tensor(device).clone()
    prim = torch.empty(pixels, dtype=torch.int32, device=device) if want_prim_id else None
    # layered jobs: the chooser's slots, saved for the backward
    layer_prim = torch.empty((_lib.MAX_LAYERS, pixels), dtype=torch.int32, device=device) if max_layers > 0 else None
    ties = torch.zeros(1, dtype=torch.int64, device=device) if count_ties else None
    jobs_dev = torch.frombuffer(bytearray(bytes(jobs)), dtype=torch.uint8).to(device)
    keep.append(jobs_dev)

    b = _lib.RastBatch()
    b.jobs = jobs_dev.data_ptr()
    b.n_jobs = n
    b.max_width, b.max_height, b.max_verts, b.max_faces = maxw, maxh, maxv, maxf
    b.shader_mask = mask
    b.total_vout, b.total_setup, b.total_pixels = vout, setup, pixels
    b.max_layers = max_layers
    P = b.pools
    for name, t in tensors.items():
        setattr(P, name, _ptr(t))
    P.zbuffer = _ptr(zbuf)
    P.canvas = _ptr(canvas)
    P.prim_id = _ptr(prim)
    P.layer_prim = _ptr(layer_prim)
    b.near_ties = _ptr(ties)
    return PackedBatch(b, keep, zbuf, canvas, prim, ties, pixel_begin,
                       {k: v for k, v in tensors.items() if v is not None}, jobs, layer_prim)


def render_plain(packed: PackedBatch, stream: Optional[torch.cuda.Stream] = None) -> None:
    """Run the plain form on a packed batch (stream-ordered; no sync)."""
    lib = _lib.load()
    b = packed.batch
    nbytes = lib.rast_plain_workspace_bytes(ctypes.byref(b))
    dev = packed.zbuffer.device
    ws = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
    packed.keep.append(ws)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    st = lib.rast_render_plain(ctypes.byref(b), ws.data_ptr(), int(nbytes), s.cuda_stream)
    _lib.check(st, "rast_render_plain")


def render_tiled(packed: PackedBatch, tile=(8, 8), bin_capacity: int = 0,
                 stream: Optional[torch.cuda.Stream] = None, small_area: int = 0,
                 warps_per_tile: int = 1) -> "_lib.RastTiledStats":
    """Run the tiled form on a packed batch; returns its bin statistics
    (reading them synchronises the stream)."""
    lib = _lib.load()
    b = packed.batch
    cfg = _lib.RastTiledConfig(int(tile[0]), int(tile[1]), int(bin_capacity), int(small_area), int(warps_per_tile))
    nbytes = lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(cfg))
    dev = packed.zbuffer.device
    ws = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=dev)
    packed.keep.append(ws)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _lib.check(lib.rast_render_tiled(ctypes.byref(b), ctypes.byref(cfg), ws.data_ptr(), int(nbytes), s.cuda_stream),
               "rast_render_tiled")
    stats = _lib.RastTiledStats()
    _lib.check(lib.rast_tiled_stats(ctypes.byref(b), ctypes.byref(cfg), ws.data_ptr(), s.cuda_stream,
                                    ctypes.byref(stats)), "rast_tiled_stats")
    return stats


def render_tiled_config(packed: PackedBatch, cfg: "_lib.RastTiledConfig",
                        stream: Optional[torch.cuda.Stream] = None) -> None:
    """Run the tiled form on a packed batch with `cfg` (stream-ordered; no sync)."""
    lib = _lib.load()
    b = packed.batch
    nbytes = int(lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(cfg)))
    if nbytes == 0:
        raise ValueError(f"tile shape {cfg.tile_w}x{cfg.tile_h} has no kernel")
    dev = packed.zbuffer.device
    ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    packed.keep.append(ws)
    s = stream if stream is not None else torch.cuda.current_stream(dev)
    _lib.check(lib.rast_render_tiled(ctypes.byref(b), ctypes.byref(cfg), ws.data_ptr(), nbytes, s.cuda_stream),
               "rast_render_tiled")


def unpack(packed: PackedBatch, specs: Sequence[JobSpec]):
    """Per-job views of the output pools: (zbuffer, canvas or None, prim_id or None)."""
    out = []
    for k, s in enumerate(specs):
        b, n = packed.pixel_begin[k], s.width * s.height
        z = packed.zbuffer[b : b + n].view(s.width, s.height)
        c = None if packed.canvas is None else packed.canvas[b * 3 : (b + n) * 3].view(s.width, s.height, 3)
        p = None if packed.prim_id is None else packed.prim_id[b : b + n].view(s.width, s.height)
        out.append((z, c, p))
    return out


__all__ = ["JobSpec", "job_from_extra", "pack", "render_plain", "render_tiled", "render_tiled_config", "unpack",
           "PackedBatch"]
