"""Renderer facade (renderer/renderer.py of jaxrenderer).

`Renderer.get_camera_image` merges the objects, builds the camera matrices,
flattens attributes per face corner and runs the Phong-reflection pipeline,
optionally after the light-space depth pass.  Host set-up is NumPy; both
passes are CUDA kernels.
"""
from __future__ import annotations

from typing import Any, NamedTuple, Optional, Sequence, Union

import numpy as np
import torch

from .geometry import Camera, _arr, normalise
from .model import MergedModel, ModelObject, merge_objects
from . import _lib
from .jobs import JobSpec, job_from_extra
from .pipeline import default_device, render_jobs
from .shaders.phong_reflection import PhongReflectionTextureExtraInput, PhongReflectionTextureShader
from .shaders.phong_reflection_shadow import (
    PhongReflectionShadowTextureExtraInput,
    PhongReflectionShadowTextureShader,
)
from .shadow import Shadow
from .types import Buffers, DtypeInfo, LightSource

F32 = np.float32


class CameraParameters(NamedTuple):
    """Camera parameters (renderer.py:46-73)."""

    viewWidth: int = 640
    viewHeight: int = 480
    viewDepth: float = 1.0
    near: float = 0.01
    far: float = 1000.0
    hfov: float = 58.0
    vfov: float = 45.0
    position: Any = np.ones(3, dtype=F32)
    target: Any = np.zeros(3, dtype=F32)
    up: Any = np.array((0.0, 0.0, 1.0), dtype=F32)


class LightParameters(NamedTuple):
    """Directional light parameters (renderer.py:76-109)."""

    direction: Any = normalise(np.array((0.57735, 0.57735, 0.57735), dtype=F32))
    colour: Any = np.ones(3, dtype=F32)
    ambient: Any = np.array((0.6, 0.6, 0.6), dtype=F32)
    diffuse: Any = np.array((0.35, 0.35, 0.35), dtype=F32)
    specular: Any = np.array((0.05, 0.05, 0.05), dtype=F32)


class ShadowParameters(NamedTuple):
    """Shadow-map parameters (renderer.py:112-133)."""

    centre: Any = np.zeros(3, dtype=F32)
    up: Any = np.array((0.0, 0.0, 1.0), dtype=F32)
    strength: Any = (np.float32(1) - np.array((0.4, 0.4, 0.4), dtype=F32)).astype(F32)
    offset: float = 0.05


def gather_rows(arr, idx) -> np.ndarray:
    """arr[idx] with jnp default gather semantics: negatives wrap once, the
    rest clamps."""
    a = np.asarray(arr)
    i = np.asarray(idx).astype(np.int64)
    n = a.shape[0]
    i = np.where(i < 0, i + n, i)
    return a[np.clip(i, 0, n - 1)]


class Renderer:
    @staticmethod
    def create_camera_from_parameters(camera: CameraParameters) -> Camera:
        """Camera matrices from parameters (renderer.py:141-196)."""
        eye = _arr(camera.position, F32)
        centre = _arr(camera.target, F32)
        up = _arr(camera.up, F32)
        view = Camera.view_matrix(eye=eye, centre=centre, up=up)
        view_inv = Camera.view_matrix_inv(eye=eye, centre=centre, up=up)
        half = np.asarray(2.0, dtype=F32)
        rad = np.asarray(np.pi / 180.0, dtype=F32)
        aspect = np.tan(np.asarray(camera.hfov, F32) * rad / half) / np.tan(np.asarray(camera.vfov, F32) * rad / half)
        projection = Camera.perspective_projection_matrix(
            fovy=camera.vfov, aspect=aspect, z_near=camera.near, z_far=camera.far
        )
        viewport = Camera.viewport_matrix(
            lowerbound=np.zeros(2, dtype=np.int32),
            dimension=np.array((camera.viewWidth, camera.viewHeight)),
            depth=np.asarray(camera.viewDepth, dtype=F32),
        )
        return Camera.create(view=view, projection=projection, viewport=viewport, view_inv=view_inv)

    @staticmethod
    def create_buffers(width: int, height: int, batch: Optional[int] = None,
                       colour_default=np.array((1.0, 1.0, 1.0), dtype=F32),
                       zbuffer_default=np.array(1, dtype=F32), device=None) -> Buffers:
        """Device buffers filled with the defaults (renderer.py:201-243)."""
        device = device if device is not None else default_device()
        lead = (batch,) if batch is not None else ()
        colour = torch.as_tensor(np.asarray(colour_default, dtype=F32).reshape(-1), device=device)
        zb = torch.full(lead + (width, height), float(np.asarray(zbuffer_default, F32)), dtype=torch.float32, device=device)
        canvas = colour.expand(lead + (width, height, colour.numel())).contiguous()
        return Buffers(zbuffer=zb, targets=(canvas,))

    @staticmethod
    def flatten_corners(model: MergedModel):
        """Per-face-corner attributes and face indices (renderer.py:277-295)."""
        faces = np.asarray(model.faces).reshape(-1)
        faces_uv = np.asarray(model.faces_uv).reshape(-1)
        position = gather_rows(_arr(model.verts, F32), faces)
        normal = gather_rows(_arr(model.norms, F32), np.asarray(model.faces_norm).reshape(-1))
        uv = gather_rows(_arr(model.uvs, F32), faces_uv)
        texture_index = gather_rows(np.asarray(model.texture_index, np.int32), faces_uv)
        face_indices = np.arange(faces.size, dtype=np.int32).reshape(np.asarray(model.faces).shape)
        return position, normal, uv, texture_index, face_indices

    @classmethod
    def _extra(cls, model: MergedModel, light: LightParameters, camera: Camera):
        position, normal, uv, texture_index, face_indices = cls.flatten_corners(model)
        light_dir = normalise(_arr(light.direction, F32))
        light_dir_eye = Camera.apply_vec(light_dir, camera.view)
        extra = PhongReflectionTextureExtraInput(
            position=position,
            normal=normal,
            uv=uv,
            light=LightSource(direction=light_dir, colour=_arr(light.colour, F32)),
            light_dir_eye=light_dir_eye,
            texture_shape=np.asarray(model.texture_shape, np.int32),
            texture_index=texture_index,
            texture_offset=np.asarray(model.offset, dtype=np.int32),
            texture=_arr(model.diffuse_map, F32),
            specular_map=_arr(model.specular_map, F32),
            ambient=_arr(light.ambient, F32),
            diffuse=_arr(light.diffuse, F32),
            specular=_arr(light.specular, F32),
        )
        return extra, face_indices

    # ------------------------------------------------------------ batching
    #
    # Every argument may carry one extra leading axis of B scenes, as under
    # jax.vmap of these calls (examples/batch_rendering.py:87-95 vmaps
    # Renderer.render over batch_models(...) and batched buffers; the
    # notebooks vmap get_camera_image over batched ModelObjects and
    # CameraParameters).  _UNBATCHED_NDIM gives each field's rank without it.

    _UNBATCHED_NDIM = {
        "MergedModel": dict(verts=2, norms=2, uvs=2, faces=2, faces_norm=2, faces_uv=2, texture_shape=2,
                            texture_index=1, double_sided=1, offset=0, diffuse_map=3, specular_map=2),
        "Model": dict(verts=2, norms=2, uvs=2, faces=2, faces_norm=2, faces_uv=2, diffuse_map=3, specular_map=2),
        "ModelObject": dict(local_scaling=1, transform=2, double_sided=0),
        "Camera": dict(view=2, projection=2, viewport=2, world_to_clip=2, world_to_eye_norm=2,
                       world_to_screen=2, view_inv=2, screen_to_world=2),
        "CameraParameters": dict(viewWidth=0, viewHeight=0, viewDepth=0, near=0, far=0, hfov=0, vfov=0,
                                 position=1, target=1, up=1),
        "LightParameters": dict(direction=1, colour=1, ambient=1, diffuse=1, specular=1),
        "ShadowParameters": dict(centre=1, up=1, strength=1, offset=0),
    }

    @classmethod
    def _batch_size(cls, *trees):
        """B when any argument carries a leading batch axis (all batched
        arguments must agree), else None."""
        sizes = set()
        for t in trees:
            if t is None:
                continue
            if isinstance(t, (list, tuple)) and not hasattr(t, "_fields"):
                for x in t:
                    b = cls._batch_size(x)
                    if b is not None:
                        sizes.add(b)
                continue
            ranks = cls._UNBATCHED_NDIM.get(type(t).__name__)
            if ranks is None:
                continue
            for name in t._fields:
                v = getattr(t, name)
                if name == "model":
                    b = cls._batch_size(v)
                    if b is not None:
                        sizes.add(b)
                elif name in ranks and np.ndim(v) == ranks[name] + 1:
                    sizes.add(int(np.shape(v)[0]))
        if len(sizes) > 1:
            raise ValueError(f"batched arguments disagree on the batch size: {sorted(sizes)}")
        return sizes.pop() if sizes else None

    @classmethod
    def _take(cls, t, b: int):
        """Scene b of a possibly batched argument (unbatched fields are shared)."""
        if t is None:
            return None
        if isinstance(t, (list, tuple)) and not hasattr(t, "_fields"):
            return [cls._take(x, b) for x in t]
        ranks = cls._UNBATCHED_NDIM.get(type(t).__name__)
        if ranks is None:
            return t
        out = {}
        for name in t._fields:
            v = getattr(t, name)
            if name == "model":
                out[name] = cls._take(v, b)
            elif name in ranks and np.ndim(v) == ranks[name] + 1:
                out[name] = v[b]
            else:
                out[name] = v
        return type(t)(**out)

    @classmethod
    def _scene_specs(cls, model: MergedModel, light: LightParameters, camera: Camera, width: int, height: int,
                     shadow_param: Optional[ShadowParameters]):
        """(DepthShader JobSpec or None, Phong-reflection JobSpec) of one
        scene, as Renderer.render issues them (renderer.py:254-385): with
        shadows, the light-space depth pass over the merged vertices into a
        map of the canvas size through the camera's viewport
        (Shadow.render_shadow_map, shadow.py:49-125), then the shadowed
        shader reading it (its shadow_map is set once the pass has run)."""
        extra, face_indices = cls._extra(model, light, camera)
        if shadow_param is None:
            main = job_from_extra(_lib.SHADER_PHONG_REFLECTION, camera, extra, width, height)
            main.faces = face_indices
            return None, main
        scam = Shadow.light_camera(_arr(light.direction, F32), camera.viewport, shadow_param.centre,
                                   shadow_param.up)
        depth = JobSpec(shader=_lib.SHADER_DEPTH, width=width, height=height, viewport=scam.viewport,
                        world_to_clip=scam.world_to_clip, world_to_eye_norm=scam.world_to_eye_norm,
                        position=_arr(model.verts, F32), faces=np.asarray(model.faces, np.int32).reshape(-1, 3),
                        depth_offset=float(np.float32(shadow_param.offset)), apply_depth_offset=True)
        shadow = Shadow(shadow_map=None, strength=_arr(shadow_param.strength, F32), camera=scam)
        sextra = PhongReflectionShadowTextureExtraInput(**extra._asdict(), shadow=shadow, camera=camera)
        main = job_from_extra(_lib.SHADER_PHONG_REFLECTION_SHADOW, camera, sextra, width, height)
        main.faces = face_indices
        return depth, main

    @classmethod
    def _render_scenes(cls, scenes, zbuffers, canvases, device):
        """Render scenes [(model, light, camera, shadow_param)] into their
        buffers: every scene's depth pass as one batch, then every scene's
        main pass as one batch.  Returns per-scene (zbuffer, canvas, prim_id)."""
        width, height = int(zbuffers[0].shape[0]), int(zbuffers[0].shape[1])
        pairs = [cls._scene_specs(m, l, c, width, height, sp) for m, l, c, sp in scenes]
        depth = [(k, d) for k, (d, _) in enumerate(pairs) if d is not None]
        if depth:
            fmax = float(DtypeInfo.create(np.float32).max)
            init = [torch.full((width, height), fmax, dtype=torch.float32, device=device)] * len(depth)
            maps, _, _, _ = render_jobs([d for _, d in depth], init, [None] * len(depth), device)
            for (k, _), smap in zip(depth, maps):
                pairs[k][1].shadow_map = smap
        mains = [m for _, m in pairs]
        return render_jobs(mains, zbuffers, canvases, device)[:3]

    @classmethod
    def render(cls, model: MergedModel, light: LightParameters, camera: Camera, buffers: Buffers,
               shadow_param: Optional[ShadowParameters] = None, loop_unroll: int = 1,
               with_ids: bool = False):
        """Render a merged model (renderer.py:254-385).  With `with_ids`
        returns (buffers, winning-primitive buffer).

        Any argument may carry a leading batch axis (the model from
        batch_models, buffers from create_buffers(batch=B), batched cameras,
        lights or shadow parameters): all B scenes then render as one
        batch per pass, and the buffers come back batched."""
        zb = buffers.zbuffer
        canvas = buffers.targets[0] if len(buffers.targets) > 0 else None
        B = cls._batch_size(model, light, camera, shadow_param)
        if B is None and np.ndim(zb) == 3:
            B = int(zb.shape[0])
        device = zb.device if isinstance(zb, torch.Tensor) else default_device()
        if B is None:
            z, c, p = cls._render_scenes([(model, light, camera, shadow_param)], [zb], [canvas], device)
            out = Buffers(zbuffer=z[0], targets=(c[0],) if c[0] is not None else ())
            return (out, p[0]) if with_ids else out
        scenes = [(cls._take(model, b), cls._take(light, b), cls._take(camera, b), cls._take(shadow_param, b))
                  for b in range(B)]
        zbs = [zb[b] if np.ndim(zb) == 3 else zb for b in range(B)]
        cvs = [None if canvas is None else (canvas[b] if np.ndim(canvas) == 4 else canvas) for b in range(B)]
        z, c, p = cls._render_scenes(scenes, zbs, cvs, device)
        out = Buffers(zbuffer=torch.stack(z), targets=(torch.stack(c),) if c[0] is not None else ())
        return (out, torch.stack(p)) if with_ids else out

    @classmethod
    def get_camera_image(cls, objects: Sequence[ModelObject], light: LightParameters,
                         camera: Union[Camera, CameraParameters], width: int, height: int,
                         colour_default=np.array((1.0, 1.0, 1.0), dtype=F32),
                         zbuffer_default=np.array(1, dtype=F32),
                         shadow_param: Optional[ShadowParameters] = None,
                         loop_unroll: int = 1) -> torch.Tensor:
        """Render objects to a (width, height, 3) canvas (renderer.py:395-476).

        Batched inputs (every ModelObject array, the camera, the light or the
        shadow parameters with a leading axis of B frames, the form the
        reference's notebooks pass to jax.vmap(get_camera_image)) give a
        (B, width, height, 3) canvas, all frames rendered as one batch; when
        the frames share their meshes (only transforms, cameras, lights and
        shadow centres change), the batch is merged on the device and its
        set-up is kept between calls (batched_api)."""
        B = cls._batch_size(objects, light, camera, shadow_param)
        if B is not None:
            from . import batched_api

            return batched_api.get_camera_image(objects, light, camera, width, height, colour_default,
                                                zbuffer_default, shadow_param, B)
        _camera = cls.create_camera_from_parameters(camera) if isinstance(camera, CameraParameters) else camera
        buffers = cls.create_buffers(width=width, height=height, colour_default=colour_default,
                                     zbuffer_default=zbuffer_default)
        model = merge_objects(objects)
        out = cls.render(model=model, light=light, camera=_camera, buffers=buffers,
                         shadow_param=shadow_param, loop_unroll=loop_unroll)
        return out.targets[0]


__all__ = ["CameraParameters", "LightParameters", "ShadowParameters", "Renderer", "gather_rows"]
