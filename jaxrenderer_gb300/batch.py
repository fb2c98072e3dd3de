"""Many scenes per call: the batched entry point of the rasteriser.

A `SceneBatch` holds N scenes in flat device pools (per-corner vertex
attributes, merged textures, one camera per scene) and renders them with one
launch sequence per pass: the light-space depth pass of every scene, then the
main pass of every scene.  This is the GPU counterpart of the reference's
`jax.jit(jax.vmap(Renderer.get_camera_image))` over scenes
(notebooks/84x84/A100.ipynb, examples/batch_rendering.py:87-95), with uneven
triangle counts per scene instead of padded batches.

`render_batch(batch, form="plain")` runs the plain per-pixel-scan kernels;
`form="tiled"` runs the binned tiled kernels (rast_tiled.cu).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _lib
from .geometry import Camera, apply_vec_rows, bmatmul, normalise, view_matrices, view_matrices_inv
from .renderer import CameraParameters, LightParameters, Renderer, ShadowParameters
from .shadow import Shadow

F32 = np.float32
JOB_DTYPE = np.dtype(_lib.RastJob)


def job_table(n: int) -> np.ndarray:
    """Zeroed structured array with the RastJob layout."""
    return np.zeros(n, dtype=JOB_DTYPE)


@dataclass
class SceneBatch:
    """N scenes, flattened per face corner, resident on one device."""

    n_scenes: int
    width: int
    height: int
    shadow_width: int
    shadow_height: int
    pools: Dict[str, torch.Tensor]
    main_jobs: np.ndarray  # RastJob table of the main pass
    shadow_jobs: Optional[np.ndarray]  # RastJob table of the depth pass, or None
    device: torch.device
    n_faces: np.ndarray = field(default=None)
    shadow_index: Optional[np.ndarray] = None  # scene -> shadow job row or -1

    @property
    def total_faces(self) -> int:
        return int(self.n_faces.sum())


def _cameras(positions: np.ndarray, params: CameraParameters, targets=None):
    """(world_to_clip, world_to_eye_norm, view) of one camera per row of
    `positions` (targets per row or params.target), each bit for bit what
    Renderer.create_camera_from_parameters gives for that camera, plus the
    shared viewport."""
    positions = np.asarray(positions, F32).reshape(-1, 3)
    cam = _lens(params)  # projection and viewport are shared
    centre = np.asarray(targets if targets is not None else params.target, F32)
    up = np.asarray(params.up, F32)
    view = view_matrices(positions, centre, up)
    view_inv = view_matrices_inv(positions, centre, up)
    w2c = bmatmul(cam.projection, view)
    w2e = np.ascontiguousarray(np.swapaxes(view_inv, -1, -2))
    return w2c, w2e, view, cam.viewport


_LENSES: dict = {}


def _lens(params: CameraParameters) -> Camera:
    """A camera of `params` (its projection and viewport, which do not depend
    on the position or target), built once per set of shared parameters."""
    key = repr(tuple(np.asarray(getattr(params, f)).tolist() for f in
                     ("viewWidth", "viewHeight", "viewDepth", "near", "far", "hfov", "vfov", "up")))
    cam = _LENSES.get(key)
    if cam is None:
        with np.errstate(all="ignore"):  # the stand-in position may be parallel to `up`: its view is unused
            cam = Renderer.create_camera_from_parameters(params._replace(position=np.array((1.0, 0.0, 0.0), F32),
                                                                         target=np.zeros(3, F32)))
        _LENSES[key] = cam
    return cam


def _light_cameras(light_direction, viewport, centres: np.ndarray, up, eye_norm: bool = True):
    """Shadow.light_camera for one centre per row: (world_to_clip,
    world_to_eye_norm), bit for bit the single-centre results.  With
    `eye_norm` False the second is None (the DepthShader the light cameras
    serve reads no normal transform)."""
    from .geometry import _arr, lu_inverse

    d = _arr(light_direction, F32)
    c = np.asarray(centres, F32).reshape(-1, 3)
    eye = c + d * F32(10.0)
    view = view_matrices(eye, c, _arr(up, F32))
    ortho = Camera.orthographic_projection_matrix(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0)
    w2c = bmatmul(ortho, view)
    w2e = np.ascontiguousarray(np.swapaxes(lu_inverse(view), -1, -2)) if eye_norm else None
    return w2c, w2e


@dataclass
class SceneTables:
    """Job tables of a flat scene batch (host only)."""

    main_jobs: np.ndarray
    shadow_jobs: Optional[np.ndarray]
    width: int
    height: int
    shadow_width: int
    shadow_height: int
    shadow_index: Optional[np.ndarray] = None  # scene -> row of shadow_jobs, -1 without a shadow pass


def scene_batch_tables(flat, width: int = 84, height: int = 84,
                       light: LightParameters = LightParameters(),
                       shadow_param: Optional[ShadowParameters] = ShadowParameters(),
                       shadow_size=(128, 128), camera_params: Optional[CameraParameters] = None,
                       shadow_mask: Optional[np.ndarray] = None, shadow_viewport: str = "map") -> SceneTables:
    """RastJob tables of a synthetic.FlatScenes batch.

    Each scene: PhongReflection(Shadow)TextureShader over its corners
    (Renderer.render, renderer.py:254-385); with `shadow_param`, a DepthShader
    pass into a shadow_size map seen through an orthographic light camera
    with viewport shadow_size (the low-level Shadow.render_shadow_map API).
    `shadow_mask` (N,) selects the scenes that get the shadow pass (all by
    default); the others render with PhongReflectionTextureShader.
    `shadow_param.centre` may hold one centre per scene (N, 3);
    `shadow_viewport="camera"` gives the depth pass the scene camera's
    viewport, as Renderer.render does (renderer.py:343-365).
    """
    n = flat.n_scenes
    T = int(getattr(flat, "tex_size", 4))
    Ts = int(getattr(flat, "spec_size", None) or T)
    params = camera_params or CameraParameters(viewWidth=width, viewHeight=height, near=0.01, far=1000.0,
                                               hfov=58.0, vfov=58.0, target=np.zeros(3, F32))
    viewport = Renderer.create_camera_from_parameters(params).viewport
    light_dir = normalise(np.asarray(light.direction, F32))

    shadow = shadow_param is not None
    mask = np.ones(n, bool) if shadow_mask is None else np.asarray(shadow_mask, bool)
    if not shadow:
        mask = np.zeros(n, bool)
    main = job_table(n)
    main["shader"] = np.where(mask, _lib.SHADER_PHONG_REFLECTION_SHADOW, _lib.SHADER_PHONG_REFLECTION)
    main["width"], main["height"] = width, height
    main["n_verts"] = 3 * flat.n_faces
    main["n_faces"] = flat.n_faces
    main["n_objects"] = flat.n_objects
    main["texture_offset"] = T
    main["vert_begin"] = flat.corner_begin
    main["face_begin"] = 0
    main["pixel_begin"] = np.arange(n, dtype=np.int64) * width * height
    main["vout_begin"] = flat.corner_begin
    main["setup_begin"] = np.concatenate([[0], np.cumsum(flat.n_faces.astype(np.int64))[:-1]])
    obj_begin = np.concatenate([[0], np.cumsum(flat.n_objects.astype(np.int64))[:-1]])
    main["texture_begin"] = obj_begin * T * T * 3
    main["specular_begin"] = obj_begin * Ts * Ts
    main["texture_shape_begin"] = obj_begin
    main["tex_w"] = T * flat.n_objects
    main["tex_h"], main["tex_c"] = T, 3
    main["spec_w"] = Ts * flat.n_objects
    main["spec_h"] = Ts
    main["viewport"] = np.broadcast_to(viewport.reshape(16), (n, 16))
    main["light_direction"] = light_dir
    main["light_colour"] = np.asarray(light.colour, F32)
    main["ambient"] = np.asarray(light.ambient, F32)
    main["diffuse"] = np.asarray(light.diffuse, F32)
    main["specular"] = np.asarray(light.specular, F32)
    shadow_jobs = None
    sw, sh = shadow_size
    if shadow:
        # shadow_viewport "map": the low-level API with a viewport of the map's
        # size; "camera": Renderer.render, the scene camera's viewport
        svp = viewport if shadow_viewport == "camera" else \
            Camera.viewport_matrix(np.zeros(2, np.int32), np.array((sw, sh)), 1.0)
        sel = np.nonzero(mask)[0]
        shadow_jobs = job_table(len(sel))
        shadow_jobs["shader"] = _lib.SHADER_DEPTH
        shadow_jobs["width"], shadow_jobs["height"] = sw, sh
        for k in ("n_verts", "n_faces", "vert_begin", "face_begin"):
            shadow_jobs[k] = main[k][sel]
        nf = shadow_jobs["n_faces"].astype(np.int64)
        nvt = shadow_jobs["n_verts"].astype(np.int64)
        shadow_jobs["setup_begin"] = np.concatenate([[0], np.cumsum(nf)[:-1]])
        shadow_jobs["vout_begin"] = np.concatenate([[0], np.cumsum(nvt)[:-1]])
        shadow_jobs["pixel_begin"] = np.arange(len(sel), dtype=np.int64) * sw * sh
        shadow_jobs["viewport"] = svp.reshape(16)
        shadow_jobs["depth_offset"] = np.float32(shadow_param.offset)
        shadow_jobs["flags"] = _lib.JOB_APPLY_DEPTH_OFFSET
        main["shadow_begin"][sel] = shadow_jobs["pixel_begin"]
        main["shadow_w"][sel], main["shadow_h"][sel] = sw, sh
        main["shadow_viewport"][sel] = svp.reshape(16)
        main["shadow_strength"][sel] = np.asarray(shadow_param.strength, F32)
    if shadow_jobs is not None and len(shadow_jobs) == 0:
        shadow_jobs = None
    index = np.full(n, -1, np.int64)
    if shadow_jobs is not None:
        index[np.nonzero(mask)[0]] = np.arange(len(shadow_jobs))
    t = SceneTables(main, shadow_jobs, width, height, sw, sh, index)
    frame_matrices(t, flat.camera_position, getattr(flat, "camera_target", None), params, light, shadow_param)
    return t


def frame_matrices(t: SceneTables, positions, targets, params: CameraParameters, light: LightParameters,
                   shadow_param: Optional[ShadowParameters]) -> SceneTables:
    """Write the per-frame matrices into job tables from scene_batch_tables
    (in place; same light, shadow set-up and scenes): the cameras at
    `positions` / `targets` (world_to_clip, world_to_eye_norm and the eye-space
    light direction of the main pass) and the light cameras at the shadow
    centres (the depth pass's matrices and the main pass's
    shadow_world_to_clip).  Each row gets the bits the per-scene set-up
    (Renderer.create_camera_from_parameters, Shadow.light_camera) gives it."""
    main = t.main_jobs
    n = len(main)
    w2c, w2e, views, _ = _cameras(positions, params, targets)
    main["world_to_clip"] = w2c.reshape(n, 16)
    main["world_to_eye_norm"] = w2e.reshape(n, 16)
    main["light_dir_eye"] = apply_vec_rows(normalise(np.asarray(light.direction, F32)), views)
    if t.shadow_jobs is not None:
        svp = t.shadow_jobs["viewport"][0].reshape(4, 4)
        centre = np.asarray(shadow_param.centre, F32)
        if centre.ndim == 2:  # one shadow centre per scene
            s_w2c, _ = _light_cameras(light.direction, svp, centre, shadow_param.up, eye_norm=False)
        else:
            scam = Shadow.light_camera(np.asarray(light.direction, F32), svp, centre, shadow_param.up)
            s_w2c = np.broadcast_to(scam.world_to_clip, (n, 4, 4))
        sel = np.nonzero(t.shadow_index >= 0)[0]
        t.shadow_jobs["world_to_clip"] = s_w2c[sel].reshape(-1, 16)
        # the DepthShader transforms no normals: its world_to_eye_norm stays the identity
        t.shadow_jobs["world_to_eye_norm"] = np.identity(4, dtype=F32).reshape(16)
        main["shadow_world_to_clip"][sel] = s_w2c[sel].reshape(-1, 16)
    return t


def flat_pools(flat, device) -> Dict[str, torch.Tensor]:
    """Device pools of a synthetic.FlatScenes batch."""

    def T(x, dt=torch.float32):
        return torch.from_numpy(np.ascontiguousarray(x)).to(device=device, dtype=dt)

    max_f = int(flat.n_faces.max())
    faces = np.arange(3 * max_f, dtype=np.int32).reshape(-1, 3)  # face f of every scene is corners 3f..3f+2
    return {
        "position": T(flat.position),
        "normal": T(flat.normal),
        "uv": T(flat.uv),
        "texture_index": T(flat.texture_index, torch.int32),
        "faces": T(faces, torch.int32),
        "texture": T(flat.texture),
        "specular_map": T(flat.specular_map),
        "texture_shape": T(_texture_shapes(flat), torch.int32),
    }


def _texture_shapes(flat) -> np.ndarray:
    ts = getattr(flat, "texture_shape", None)
    if ts is not None:
        return np.asarray(ts, np.int32).reshape(-1, 2)
    return np.tile(np.array([[getattr(flat, "tex_size", 4)] * 2], np.int32), (int(flat.n_objects.sum()), 1))


def scene_batch_from_flat(flat, width: int = 84, height: int = 84,
                          light: LightParameters = LightParameters(),
                          shadow_param: Optional[ShadowParameters] = ShadowParameters(),
                          shadow_size=(128, 128), device=None,
                          camera_params: Optional[CameraParameters] = None,
                          shadow_mask: Optional[np.ndarray] = None) -> SceneBatch:
    """Upload a synthetic.FlatScenes batch and build its job tables."""
    device = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    t = scene_batch_tables(flat, width, height, light, shadow_param, shadow_size, camera_params, shadow_mask)
    lib = _lib.load()
    for tbl in (t.main_jobs, t.shadow_jobs):
        if tbl is None:
            continue
        for k in range(min(len(tbl), 4)):
            job = _lib.RastJob.from_buffer_copy(tbl[k].tobytes())
            _lib.check(lib.rast_validate_job(ctypes.byref(job)), f"job {k}")
    return SceneBatch(flat.n_scenes, width, height, t.shadow_width, t.shadow_height, flat_pools(flat, device),
                      t.main_jobs, t.shadow_jobs, device, flat.n_faces, t.shadow_index)


def scene_batch_from_instances(inst, width: int = 84, height: int = 84,
                               light: LightParameters = LightParameters(),
                               shadow_param: Optional[ShadowParameters] = ShadowParameters(),
                               shadow_size=(128, 128), device=None,
                               camera_params: Optional[CameraParameters] = None,
                               shadow_mask: Optional[np.ndarray] = None, shadow_viewport: str = "map"):
    """A SceneBatch of an instancing.InstancedScenes batch whose per-corner
    pools are built on the device; returns (SceneBatch, DeviceMerge) after
    one merge.  Later frames: `merge.merge(transforms, local_scaling)` then
    render again."""
    from .instancing import DeviceMerge, instanced_pools

    device = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    shell = inst.shell()
    t = scene_batch_tables(shell, width, height, light, shadow_param, shadow_size, camera_params, shadow_mask,
                           shadow_viewport)
    pools = instanced_pools(inst, device)
    merge = DeviceMerge(inst, pools, device)
    merge.merge()
    sb = SceneBatch(inst.n_scenes, width, height, t.shadow_width, t.shadow_height, pools, t.main_jobs,
                    t.shadow_jobs, device, shell.n_faces, t.shadow_index)
    return sb, merge


def set_layers(sb: SceneBatch, layers: int, mixer: int = _lib.MIX_NEAREST, opacity=1.0,
               background=(0.0, 0.0, 0.0)) -> None:
    """Main-pass primitive_chooser / mix hooks of every scene of `sb`
    (rast_gb300.h, RastMixer): the `layers` nearest candidates per pixel,
    blended by `mixer` with `opacity` (one value, or one per scene) over
    `background`.  Takes effect for runners created afterwards; the depth
    pass keeps the default chooser."""
    if not 0 <= int(layers) <= _lib.MAX_LAYERS:
        raise ValueError(f"layers must be 0..{_lib.MAX_LAYERS}")
    if mixer not in (_lib.MIX_NEAREST, _lib.MIX_OVER) or (mixer == _lib.MIX_OVER and layers == 0):
        raise ValueError("mixer must be MIX_NEAREST, or MIX_OVER with layers >= 1")
    t = sb.main_jobs
    if layers > 0 and np.any(t["shader"] == _lib.SHADER_DEPTH):
        raise ValueError("the DEPTH shader takes the default chooser only")
    t["layers"] = int(layers)
    t["mixer"] = int(mixer)
    t["opacity"] = np.broadcast_to(np.asarray(opacity, F32), (len(t),))
    t["background"] = np.broadcast_to(np.asarray(background, F32), (3,))


def scene_batch_from_specs(specs, device=None) -> SceneBatch:
    """A SceneBatch of N independent single-pass jobs (same size and shader,
    no shadow pass) from JobSpecs, e.g. N differentiable scenes."""
    from .jobs import pack

    device = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    W, H = specs[0].width, specs[0].height
    if any(s.width != W or s.height != H for s in specs):
        raise ValueError("scene_batch_from_specs needs equal sizes")
    z = [np.ones((W, H), F32)] * len(specs)
    packed = pack(specs, z, [None] * len(specs), device, want_prim_id=False)
    jobs = np.frombuffer(bytes(packed.jobs), dtype=JOB_DTYPE).copy()
    n_faces = jobs["n_faces"].astype(np.int32)
    return SceneBatch(len(specs), W, H, 0, 0, packed.pools, jobs, None, device, n_faces)


def scene_job_specs(flat, tables, s: int):
    """The pipeline.render calls scene `s` of a flat batch makes, as JobSpecs
    with host arrays: (depth pass or None, main pass)."""
    from .jobs import JobSpec

    m = tables.main_jobs[s]
    T = int(getattr(flat, "tex_size", 4))
    Ts = int(getattr(flat, "spec_size", None) or T)
    cb, F = int(flat.corner_begin[s]), int(flat.n_faces[s])
    no = int(flat.n_objects[s])
    ob = int(np.sum(flat.n_objects[:s], dtype=np.int64))
    faces = np.arange(3 * F, dtype=np.int32).reshape(F, 3)
    rows = slice(cb, cb + 3 * F)
    main = JobSpec(shader=int(m["shader"]), width=int(m["width"]), height=int(m["height"]),
                   viewport=m["viewport"].reshape(4, 4), world_to_clip=m["world_to_clip"].reshape(4, 4),
                   world_to_eye_norm=m["world_to_eye_norm"].reshape(4, 4), position=flat.position[rows],
                   faces=faces)
    main.normal = flat.normal[rows]
    main.uv = flat.uv[rows]
    main.texture_index = flat.texture_index[rows]
    main.texture = flat.texture[ob * T : (ob + no) * T]
    main.specular_map = flat.specular_map[ob * Ts : (ob + no) * Ts]
    main.texture_shape = _texture_shapes(flat)[ob : ob + no]
    main.texture_offset = T
    for k in ("light_direction", "light_colour", "light_dir_eye", "ambient", "diffuse", "specular"):
        setattr(main, k, np.asarray(m[k], F32))
    main.layers, main.mixer = int(m["layers"]), int(m["mixer"])
    main.opacity, main.background = float(m["opacity"]), np.asarray(m["background"], F32)
    depth = None
    index = getattr(tables, "shadow_index", None)
    srow = s if index is None else int(index[s])
    if tables.shadow_jobs is not None and srow >= 0:
        d = tables.shadow_jobs[srow]
        depth = JobSpec(shader=_lib.SHADER_DEPTH, width=int(d["width"]), height=int(d["height"]),
                        viewport=d["viewport"].reshape(4, 4), world_to_clip=d["world_to_clip"].reshape(4, 4),
                        world_to_eye_norm=d["world_to_eye_norm"].reshape(4, 4), position=flat.position[rows],
                        faces=faces, depth_offset=float(d["depth_offset"]), apply_depth_offset=True)
        main.shadow_viewport = m["shadow_viewport"].reshape(4, 4)
        main.shadow_world_to_clip = m["shadow_world_to_clip"].reshape(4, 4)
        main.shadow_strength = np.asarray(m["shadow_strength"], F32)
    return depth, main


def _rast_batch(jobs: np.ndarray, pools: Dict[str, torch.Tensor], zbuffer: torch.Tensor,
                canvas: Optional[torch.Tensor], prim_id: Optional[torch.Tensor], ties, keep: list):
    jt = torch.from_numpy(jobs.view(np.uint8).copy()).to(zbuffer.device)
    keep.append(jt)
    keep.append(("jobs", id(jobs), jt))
    b = _lib.RastBatch()
    b.jobs = jt.data_ptr()
    b.n_jobs = len(jobs)
    b.max_width = int(jobs["width"].max())
    b.max_height = int(jobs["height"].max())
    b.max_verts = int(jobs["n_verts"].max())
    b.max_faces = int(jobs["n_faces"].max())
    b.shader_mask = int(np.bitwise_or.reduce(1 << jobs["shader"].astype(np.int64)))
    b.total_vout = int(jobs["n_verts"].astype(np.int64).sum())
    b.total_setup = int(jobs["n_faces"].astype(np.int64).sum())
    b.total_pixels = int((jobs["width"].astype(np.int64) * jobs["height"]).sum())
    b.max_layers = max(int(jobs["layers"].max()), 0)
    P = b.pools
    for name, t in pools.items():
        setattr(P, name, t.data_ptr())
    P.zbuffer = zbuffer.data_ptr()
    P.canvas = canvas.data_ptr() if canvas is not None else None
    P.prim_id = prim_id.data_ptr() if prim_id is not None else None
    b.near_ties = ties.data_ptr() if ties is not None else None
    return b


@dataclass
class BatchOutputs:
    canvas: torch.Tensor  # (N, W, H, 3)
    zbuffer: torch.Tensor  # (N, W, H)
    prim_id: Optional[torch.Tensor]  # (N, W, H)
    shadow_map: Optional[torch.Tensor]  # (N, Ws, Hs)
    shadow_prim_id: Optional[torch.Tensor]
    near_ties: Optional[torch.Tensor]


class BatchRunner:
    """Reusable outputs + workspaces for repeated renders of one SceneBatch.

    form="plain": per-pixel scan over every primitive (rast_render_plain);
    form="tiled": binned tiles (rast_render_tiled) with `tiled_config`
    (one RastTiledConfig for both passes, or a {"shadow" / "main": config}
    dict) from the autotuner where not given.
    `capture()` records one full render (buffer reset, depth pass, main pass)
    into a CUDA graph that `replay()` re-issues with a single launch.
    """

    def __init__(self, sb: SceneBatch, form: str = "plain", want_prim_id: bool = True, count_ties: bool = False,
                 tiled_config=None, overlap_passes: bool = True):
        self.sb = sb
        self.form = form
        self.overlap_passes = overlap_passes
        dev = sb.device
        n, W, H = sb.n_scenes, sb.width, sb.height
        self.canvas = torch.empty((n, W, H, 3), dtype=torch.float32, device=dev)
        self.zbuffer = torch.empty((n, W, H), dtype=torch.float32, device=dev)
        self.prim_id = torch.empty((n, W, H), dtype=torch.int32, device=dev) if want_prim_id else None
        self.ties = torch.zeros(1, dtype=torch.int64, device=dev) if count_ties else None
        self.shadow_ties = torch.zeros(1, dtype=torch.int64, device=dev) if count_ties else None
        self.shadow_map = None
        self.shadow_prim = None
        self.keep = []
        self.graph = None
        self._colour = torch.ones(3, dtype=torch.float32, device=dev)
        lib = _lib.load()
        self.lib = lib
        if sb.shadow_jobs is not None:
            self.shadow_map = torch.empty((len(sb.shadow_jobs), sb.shadow_width, sb.shadow_height),
                                          dtype=torch.float32, device=dev)
            self.shadow_prim = torch.empty_like(self.shadow_map, dtype=torch.int32) if want_prim_id else None
            self.shadow_batch = _rast_batch(sb.shadow_jobs, sb.pools, self.shadow_map, None, self.shadow_prim,
                                            self.shadow_ties, self.keep)
            self.shadow_jobs_dev = self.keep[-1][2]  # device copy of the depth pass's job table (uint8)
            pools = dict(sb.pools)
            pools["shadow_map"] = self.shadow_map
        else:
            self.shadow_batch = None
            pools = sb.pools
        self.main_batch = _rast_batch(sb.main_jobs, pools, self.zbuffer, self.canvas, self.prim_id, self.ties, self.keep)
        # layered jobs: the chooser's slots, saved for the backward (RastPools.layer_prim)
        self.layer_prim = None
        if self.main_batch.max_layers > 0:
            self.layer_prim = torch.empty((_lib.MAX_LAYERS, n * W * H), dtype=torch.int32, device=dev)
            self.main_batch.pools.layer_prim = self.layer_prim.data_ptr()
        self.main_jobs_dev = self.keep[-1][2]  # device copy of the main job table (uint8)
        self.pools = pools
        self.configs = {}
        if form == "tiled":
            from .autotune import tiled_config_for

            for name, b, tbl in (("shadow", self.shadow_batch, sb.shadow_jobs), ("main", self.main_batch, sb.main_jobs)):
                if b is None:
                    continue
                # one config for both passes, a {pass name: config} dict, or None (the autotuner's)
                cfg = tiled_config.get(name) if isinstance(tiled_config, dict) else tiled_config
                self.configs[name] = cfg if cfg is not None else tiled_config_for(self, name, b, tbl)
        self.ws = {}
        for name, b in (("shadow", self.shadow_batch), ("main", self.main_batch)):
            if b is None:
                continue
            nbytes = int(self._ws_bytes(name, b))
            self.ws[name] = (torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev), nbytes)

    def batches(self):
        return [(n, b) for n, b in (("shadow", self.shadow_batch), ("main", self.main_batch)) if b is not None]

    def _cfg(self, name):
        c = self.configs.get(name)
        return ctypes.byref(c) if c is not None else None

    def _ws_bytes(self, name, b) -> int:
        if self.form == "plain":
            return self.lib.rast_plain_workspace_bytes(ctypes.byref(b))
        return self.lib.rast_tiled_workspace_bytes(ctypes.byref(b), self._cfg(name))

    def launch(self, name, stream_handle, profile=None, phase: int = 3) -> None:
        """Render pass `name` on the stream; `phase` (tiled form) selects
        rast_render_tiled_phase's coverage (1) or shade (2) half, 3 both."""
        b = self.shadow_batch if name == "shadow" else self.main_batch
        buf, nbytes = self.ws[name]
        if self.form == "tiled" and phase != 3 and profile is None:
            st = self.lib.rast_render_tiled_phase(ctypes.byref(b), self._cfg(name), buf.data_ptr(), nbytes,
                                                  stream_handle, int(phase))
            _lib.check(st, "rast_render_tiled_phase")
            return
        if self.form == "plain":
            if profile is None:
                st = self.lib.rast_render_plain(ctypes.byref(b), buf.data_ptr(), nbytes, stream_handle)
            else:
                st = self.lib.rast_render_plain_profiled(ctypes.byref(b), buf.data_ptr(), nbytes, stream_handle,
                                                         ctypes.byref(profile))
        else:
            if profile is None:
                st = self.lib.rast_render_tiled(ctypes.byref(b), self._cfg(name), buf.data_ptr(), nbytes, stream_handle)
            else:
                st = self.lib.rast_render_tiled_profiled(ctypes.byref(b), self._cfg(name), buf.data_ptr(), nbytes,
                                                         stream_handle, ctypes.byref(profile))
        _lib.check(st, f"rast_render_{self.form}")

    def set_job_tables(self, main_jobs: np.ndarray, shadow_jobs: Optional[np.ndarray] = None,
                       stream: Optional[torch.cuda.Stream] = None) -> None:
        """Replace the device job tables with new ones of the same jobs (new
        matrices and light terms; sizes, offsets and shaders unchanged, so
        the workspaces and tiled configs stay valid).  Stream-ordered."""
        s = stream if stream is not None else torch.cuda.current_stream(self.sb.device)
        staging = self.__dict__.setdefault("_job_staging", {})
        for name, dev, tbl in (("main", self.main_jobs_dev, main_jobs),
                               ("shadow", getattr(self, "shadow_jobs_dev", None), shadow_jobs)):
            if dev is None or tbl is None:
                continue
            host = np.ascontiguousarray(tbl).view(np.uint8).reshape(-1)
            if host.size != dev.numel():
                raise ValueError("set_job_tables: the new table has another number of jobs")
            buf, done = staging.get(name, (None, None))
            if buf is None:
                buf = torch.empty(host.size, dtype=torch.uint8, pin_memory=True)
            elif done is not None:
                done.synchronize()  # the previous copy out of this pinned buffer has finished
            buf.numpy()[:] = host
            with torch.cuda.stream(s):
                dev.copy_(buf, non_blocking=True)
                done = torch.cuda.Event()
                done.record(s)
            staging[name] = (buf, done)

    def job_floats(self) -> torch.Tensor:
        """The main pass's device job table viewed as (n_jobs, sizeof(RastJob)/4)
        float32, for in-place updates of per-job matrices and light terms."""
        return self.main_jobs_dev.view(torch.float32).view(self.sb.n_scenes, -1)

    def grad_buffers(self) -> Dict[str, torch.Tensor]:
        """Zeroed gradient arrays matching the batch's pools (for backward(out=...))."""
        dev = self.sb.device
        P = self.pools
        g = {k: torch.zeros_like(P[k]) for k in ("position", "normal", "colour", "texture", "specular_map",
                                                 "normal_map") if k in P}
        g["job_params"] = torch.zeros((self.sb.n_scenes, _lib.NPARAM), dtype=torch.float32, device=dev)
        return g

    def backward(self, grad_canvas: Optional[torch.Tensor], grad_zbuffer: Optional[torch.Tensor] = None,
                 stream: Optional[torch.cuda.Stream] = None,
                 out: Optional[Dict[str, torch.Tensor]] = None, profile=None,
                 accumulate: bool = False) -> Dict[str, torch.Tensor]:
        """Gradients of the last run() of the main pass (rast_backward):
        per-vertex position/normal, per-texel texture/specular exponent and
        per-scene camera/light terms (RAST_GRAD_* layout, (N, 56)).  With
        `out` (from grad_buffers()) the arrays are zeroed and reused; with
        `accumulate` as well the gradients are added to what `out` holds
        (gradient accumulation over several renders)."""
        gc = grad_canvas.contiguous() if grad_canvas is not None else None
        gz = grad_zbuffer.contiguous() if grad_zbuffer is not None else None

        def call(args):
            if profile is None:
                return self.lib.rast_backward(args[0], gc.data_ptr() if gc is not None else None, *args[1:])
            return self.lib.rast_backward_profiled(args[0], gc.data_ptr() if gc is not None else None, *args[1:],
                                                   ctypes.byref(profile))

        return self._backward(call, gz, stream, out, accumulate, "rast_backward")

    def backward_mse(self, target: torch.Tensor, scale: Optional[float] = None,
                     grad_zbuffer: Optional[torch.Tensor] = None, stream: Optional[torch.cuda.Stream] = None,
                     out: Optional[Dict[str, torch.Tensor]] = None,
                     accumulate: bool = False) -> Dict[str, torch.Tensor]:
        """Gradients of the mean-squared-error loss (scale / 2) * sum((canvas
        - target)^2) of the last run() (rast_backward_mse): dL/dcanvas =
        (canvas - target) * scale is formed inside the backward from the
        rendered canvas, with no gradient image.  `scale` defaults to 2 /
        canvas.numel(), the gradient of the mean.  The result equals
        backward((canvas - target) * scale) up to the order of the atomic
        sums; `out` and `accumulate` as in backward()."""
        if target.shape != self.canvas.shape:
            raise ValueError(f"target shape {tuple(target.shape)} != canvas shape {tuple(self.canvas.shape)}")
        tg = target.to(dtype=torch.float32).contiguous()
        sc = float(2.0 / self.canvas.numel() if scale is None else scale)
        gz = grad_zbuffer.contiguous() if grad_zbuffer is not None else None

        def call(args):
            return self.lib.rast_backward_mse(args[0], tg.data_ptr(), sc, *args[1:])

        return self._backward(call, gz, stream, out, accumulate, "rast_backward_mse")

    def _backward(self, call, gz, stream, out, accumulate, name) -> Dict[str, torch.Tensor]:
        if self.prim_id is None:
            raise RuntimeError("backward needs the winning-primitive buffer: build the runner with want_prim_id=True")
        dev = self.sb.device
        if out is None:
            g = self.grad_buffers()
        else:
            g = out
            if not accumulate:
                for t in g.values():
                    t.zero_()
        gp = _lib.RastGradPools()
        for k, t in g.items():
            setattr(gp, k, t.data_ptr())
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        nbytes = int(self.lib.rast_backward_workspace_bytes(ctypes.byref(self.main_batch)))
        if getattr(self, "_bwd_ws", None) is None or self._bwd_ws.numel() < nbytes:
            self._bwd_ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev)
        args = (ctypes.byref(self.main_batch), gz.data_ptr() if gz is not None else None, ctypes.byref(gp),
                self._bwd_ws.data_ptr(), nbytes, s.cuda_stream)
        _lib.check(call(args), name)
        return g

    def stats(self, name="main"):
        """Bin statistics of the last tiled render of pass `name`."""
        b = self.shadow_batch if name == "shadow" else self.main_batch
        out = _lib.RastTiledStats()
        buf, _ = self.ws[name]
        s = torch.cuda.current_stream(self.sb.device)
        _lib.check(self.lib.rast_tiled_stats(ctypes.byref(b), self._cfg(name), buf.data_ptr(), s.cuda_stream,
                                             ctypes.byref(out)), "rast_tiled_stats")
        return out

    def set_colour_default(self, colour) -> None:
        """Canvas value of pixels no primitive writes (Renderer.create_buffers'
        colour_default); run() resets the canvases to it."""
        self._colour.copy_(torch.as_tensor(np.asarray(colour, F32).reshape(-1)[:3]))

    def _reset(self, zbuffer_default: float):
        self.zbuffer.fill_(zbuffer_default)
        self.canvas.copy_(self._colour.expand_as(self.canvas))
        if self.shadow_map is not None:
            self.shadow_map.fill_(float(np.finfo(np.float32).max))

    def run(self, stream: Optional[torch.cuda.Stream] = None, zbuffer_default: float = 1.0) -> BatchOutputs:
        """Reset the buffers to their defaults and render every scene on
        `stream`: the depth pass, then the main pass.  In the tiled form with
        `overlap_passes`, the depth pass runs on a side stream beside the main
        pass's coverage phase (which reads no shadow map), and the main
        pass's shading waits for both: a fork and a join, which a CUDA graph
        capture records as two branches."""
        s = stream if stream is not None else torch.cuda.current_stream(self.sb.device)
        with torch.cuda.stream(s):
            self._reset(zbuffer_default)
            if self.form == "tiled" and self.shadow_batch is not None and self.overlap_passes:
                side = self._side_stream()
                side.wait_stream(s)
                with torch.cuda.stream(side):
                    torch.cuda.nvtx.range_push("shadow pass")
                    self.launch("shadow", side.cuda_stream)
                    torch.cuda.nvtx.range_pop()
                torch.cuda.nvtx.range_push("main pass")
                self.launch("main", s.cuda_stream, phase=_lib.PHASE_COVERAGE)
                s.wait_stream(side)
                self.launch("main", s.cuda_stream, phase=_lib.PHASE_SHADE)
                torch.cuda.nvtx.range_pop()
            else:
                for name, _ in self.batches():
                    torch.cuda.nvtx.range_push(f"{name} pass")
                    self.launch(name, s.cuda_stream)
                    torch.cuda.nvtx.range_pop()
        return self.outputs()

    def _side_stream(self) -> torch.cuda.Stream:
        if getattr(self, "_side", None) is None:
            self._side = torch.cuda.Stream(self.sb.device)
        return self._side

    def outputs(self) -> BatchOutputs:
        return BatchOutputs(self.canvas, self.zbuffer, self.prim_id, self.shadow_map, self.shadow_prim, self.ties)

    def capture(self) -> None:
        """Record run() into a CUDA graph (one launch per replay)."""
        dev = self.sb.device
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        self.run(side)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(torch.cuda.current_stream(dev))
        self.graph = g

    def replay(self) -> BatchOutputs:
        self.graph.replay()
        return self.outputs()


class MultiRunner:
    """Several SceneBatches (e.g. one per resolution class of a mixed batch),
    each with its own BatchRunner and autotuned tiled config, rendered in
    order on one stream; `capture()` records all of them into ONE CUDA graph
    so a replay re-issues the whole mixed batch with a single launch."""

    def __init__(self, batches: Sequence[SceneBatch], form: str = "tiled", want_prim_id: bool = True,
                 tiled_config=None):
        if not batches:
            raise ValueError("MultiRunner needs at least one SceneBatch")
        self.runners = [BatchRunner(sb, form=form, want_prim_id=want_prim_id, tiled_config=tiled_config)
                        for sb in batches]
        self.form = form
        self.device = batches[0].device
        self.graph = None

    @property
    def n_scenes(self) -> int:
        return sum(r.sb.n_scenes for r in self.runners)

    def run(self, stream: Optional[torch.cuda.Stream] = None) -> List[BatchOutputs]:
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        return [r.run(s) for r in self.runners]

    def capture(self) -> None:
        dev = self.device
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        self.run(side)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(torch.cuda.current_stream(dev))
        self.graph = g

    def replay(self) -> List[BatchOutputs]:
        self.graph.replay()
        return [r.outputs() for r in self.runners]

    def grad_buffers(self) -> List[Dict[str, torch.Tensor]]:
        return [r.grad_buffers() for r in self.runners]

    def backward(self, grad_canvases: Sequence[torch.Tensor], out=None,
                 stream: Optional[torch.cuda.Stream] = None, accumulate: bool = False) -> List[Dict[str, torch.Tensor]]:
        outs = out if out is not None else [None] * len(self.runners)
        return [r.backward(g, stream=stream, out=o, accumulate=accumulate)
                for r, g, o in zip(self.runners, grad_canvases, outs)]

    def backward_mse(self, targets: Sequence[torch.Tensor], scales: Optional[Sequence[float]] = None, out=None,
                     stream: Optional[torch.cuda.Stream] = None,
                     accumulate: bool = False) -> List[Dict[str, torch.Tensor]]:
        """BatchRunner.backward_mse per group (the loss's scale per group:
        2 / that group's canvas size by default)."""
        outs = out if out is not None else [None] * len(self.runners)
        scs = scales if scales is not None else [None] * len(self.runners)
        return [r.backward_mse(t, c, stream=stream, out=o, accumulate=accumulate)
                for r, t, c, o in zip(self.runners, targets, scs, outs)]


class InstancedPipeline:
    """Serving loop for instanced scenes (meshes resident, transforms per
    frame), double-buffered: two SceneBatches share the tables but own their
    per-corner pools, canvases and captured render graphs, so frame k + 1's
    host -> device transform copy and device merge (rast_merge_objects) run
    on a merge stream while frame k renders, and frame k's canvases go to host
    memory on a copy stream while frame k + 1 renders.

        pipe = InstancedPipeline(instances, 84, 84, shadow_size=(128, 128))
        for k, (tr, sc) in enumerate(frames):        # pinned host tensors
            pipe.frame(tr, sc, out=host_canvases[k % 2])
        pipe.synchronize()

    `frame()` only enqueues work: host inputs must stay unchanged, and a
    host buffer passed as `out` is complete, once `done_event()` of that
    frame has been reached.  Arguments after `inst` are those of
    scene_batch_from_instances, plus the runner's form and tiled config and
    `prepare`, called on each SceneBatch before its runner is built (e.g.
    set_layers)."""

    def __init__(self, inst, width: int = 84, height: int = 84, light: LightParameters = LightParameters(),
                 shadow_param: Optional[ShadowParameters] = ShadowParameters(), shadow_size=(128, 128),
                 device=None, camera_params: Optional[CameraParameters] = None,
                 shadow_mask: Optional[np.ndarray] = None, shadow_viewport: str = "map", form: str = "tiled",
                 tiled_config=None, prepare=None):
        self.device = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.sets = []
        for _ in range(2):
            sb, merge = scene_batch_from_instances(inst, width, height, light, shadow_param, shadow_size,
                                                   self.device, camera_params, shadow_mask, shadow_viewport)
            if prepare is not None:
                prepare(sb)
            runner = BatchRunner(sb, form=form, want_prim_id=False, tiled_config=tiled_config)
            if form == "tiled":
                runner.capture()
            self.sets.append((sb, merge, runner))
        # the render stream takes precedence: the merge fills the SM
        # resources the render's kernels leave free
        self.merge_stream = torch.cuda.Stream(self.device, priority=0)
        self.render_stream = torch.cuda.Stream(self.device, priority=-1)
        self.copy_stream = torch.cuda.Stream(self.device)
        self._rendered = [None, None]  # set b's pools / canvas are in use until these
        self._copied = [None, None]
        self.k = 0

    def canvas(self, b: int) -> torch.Tensor:
        return self.sets[b][2].canvas

    def start_after(self, event: torch.cuda.Event) -> None:
        """Make the pipeline's streams wait for `event` (e.g. a timing start)."""
        for s in (self.merge_stream, self.render_stream, self.copy_stream):
            s.wait_event(event)

    def frame(self, transforms, local_scaling, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """Enqueue one frame: transforms (I, 4, 4) and local scalings (I, 3)
        (host or device), merged and rendered into set k % 2; with `out`
        (a pinned host tensor of the canvas shape) the canvases are copied
        there.  Returns the set's device canvases."""
        b = self.k % 2
        self.k += 1
        sb, merge, runner = self.sets[b]
        if self._rendered[b] is not None:  # frame k - 2 read these pools
            self.merge_stream.wait_event(self._rendered[b])
        merge.merge(transforms, local_scaling, self.merge_stream)
        merged = torch.cuda.Event()
        merged.record(self.merge_stream)
        self.render_stream.wait_event(merged)
        if self._copied[b] is not None:  # frame k - 2's canvases left for the host
            self.render_stream.wait_event(self._copied[b])
        if runner.graph is not None:
            with torch.cuda.stream(self.render_stream):
                runner.graph.replay()
        else:
            runner.run(self.render_stream)
        rendered = torch.cuda.Event()
        rendered.record(self.render_stream)
        self._rendered[b] = rendered
        copied = rendered
        if out is not None:
            self.copy_stream.wait_event(rendered)
            with torch.cuda.stream(self.copy_stream):
                out.copy_(runner.canvas, non_blocking=True)
            copied = torch.cuda.Event()
            copied.record(self.copy_stream)
        self._copied[b] = copied
        return runner.canvas

    def done_event(self) -> Optional[torch.cuda.Event]:
        """The last enqueued frame's end (its host copy when it had one)."""
        return self._copied[(self.k - 1) % 2] if self.k else None

    def pending(self) -> List[torch.cuda.Event]:
        return [e for e in self._copied if e is not None]

    def synchronize(self) -> None:
        for e in self.pending():
            e.synchronize()


def mixed_scene_batches(flat, resolutions: np.ndarray, classes: Sequence[Tuple[int, int]],
                        shadow_mask: Optional[np.ndarray] = None, light: LightParameters = LightParameters(),
                        shadow_param: Optional[ShadowParameters] = ShadowParameters(), device=None,
                        camera_params: Optional[CameraParameters] = None):
    """Split a FlatScenes batch by resolution class: scene s renders at
    classes[resolutions[s]].  Scenes with shadow_mask[s] get the depth pass
    (a map of their own canvas size, as Renderer.render makes it,
    renderer.py:343-365) and PhongReflectionShadowTextureShader, the others
    PhongReflectionTextureShader.  Returns [(scene indices, SceneBatch)] per
    non-empty class, in class order."""
    from .synthetic import flat_subset

    res = np.asarray(resolutions)
    mask = np.ones(flat.n_scenes, bool) if shadow_mask is None else np.asarray(shadow_mask, bool)
    out = []
    for c, (w, h) in enumerate(classes):
        idx = np.nonzero(res == c)[0]
        if idx.size == 0:
            continue
        sub = flat_subset(flat, idx)
        prm = None
        if camera_params is not None:
            prm = camera_params._replace(viewWidth=w, viewHeight=h)
        sb = scene_batch_from_flat(sub, w, h, light, shadow_param, (w, h), device, prm, mask[idx])
        out.append((idx, sb))
    return out


def render_batch(sb: SceneBatch, form: str = "plain", want_prim_id: bool = True) -> BatchOutputs:
    """Render every scene of `sb` (see BatchRunner)."""
    return BatchRunner(sb, form=form, want_prim_id=want_prim_id).run()


__all__ = ["SceneBatch", "SceneTables", "scene_batch_tables", "scene_batch_from_flat", "scene_batch_from_specs",
           "set_layers", "InstancedPipeline",
           "scene_job_specs", "MultiRunner", "mixed_scene_batches", "scene_batch_from_instances",
           "flat_pools", "render_batch", "BatchRunner", "BatchOutputs", "job_table"]
