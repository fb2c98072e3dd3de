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
from .pipeline import default_device, render_with_ids
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

    @classmethod
    def render(cls, model: MergedModel, light: LightParameters, camera: Camera, buffers: Buffers,
               shadow_param: Optional[ShadowParameters] = None, loop_unroll: int = 1,
               with_ids: bool = False):
        """Render a merged model (renderer.py:254-385).  With `with_ids`
        returns (buffers, winning-primitive buffer)."""
        extra, face_indices = cls._extra(model, light, camera)
        if shadow_param is None:
            out, ids, _ = render_with_ids(camera, PhongReflectionTextureShader, buffers, face_indices, extra)
            return (out, ids) if with_ids else out
        zb = buffers.zbuffer
        fmax = float(DtypeInfo.create(np.float32).max)
        shadow_map = torch.full(tuple(zb.shape), fmax, dtype=torch.float32,
                                device=zb.device if isinstance(zb, torch.Tensor) else default_device())
        shadow = Shadow.render_shadow_map(
            shadow_map=shadow_map,
            verts=_arr(model.verts, F32),
            faces=np.asarray(model.faces, np.int32),
            light_direction=_arr(light.direction, F32),
            viewport_matrix=camera.viewport,
            centre=shadow_param.centre,
            up=shadow_param.up,
            strength=shadow_param.strength,
            offset=shadow_param.offset,
            loop_unroll=loop_unroll,
        )
        _extra = PhongReflectionShadowTextureExtraInput(**extra._asdict(), shadow=shadow, camera=camera)
        out, ids, _ = render_with_ids(camera, PhongReflectionShadowTextureShader, buffers, face_indices, _extra)
        return (out, ids) if with_ids else out

    @classmethod
    def get_camera_image(cls, objects: Sequence[ModelObject], light: LightParameters,
                         camera: Union[Camera, CameraParameters], width: int, height: int,
                         colour_default=np.array((1.0, 1.0, 1.0), dtype=F32),
                         zbuffer_default=np.array(1, dtype=F32),
                         shadow_param: Optional[ShadowParameters] = None,
                         loop_unroll: int = 1) -> torch.Tensor:
        """Render objects to a (width, height, 3) canvas (renderer.py:395-476)."""
        _camera = cls.create_camera_from_parameters(camera) if isinstance(camera, CameraParameters) else camera
        buffers = cls.create_buffers(width=width, height=height, colour_default=colour_default,
                                     zbuffer_default=zbuffer_default)
        model = merge_objects(objects)
        out = cls.render(model=model, light=light, camera=_camera, buffers=buffers,
                         shadow_param=shadow_param, loop_unroll=loop_unroll)
        return out.targets[0]


__all__ = ["CameraParameters", "LightParameters", "ShadowParameters", "Renderer", "gather_rows"]
