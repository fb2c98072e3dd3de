"""Shadow map from the light's point of view (renderer/shadow.py:27-153)."""
from __future__ import annotations

from typing import Any, NamedTuple

import numpy as np
import torch

from . import _lib
from . import jobs as _jobs
from .geometry import Camera, _arr
from .pipeline import render_job


class Shadow(NamedTuple):
    """Shadow map of one parallel light (shadow.py:27-38)."""

    shadow_map: Any  # (Ws, Hs) device tensor
    strength: Any  # (3,)
    camera: Camera  # world -> shadow map screen space

    @staticmethod
    def light_camera(light_direction, viewport_matrix, centre, up, distance: float = 10.0) -> Camera:
        """Orthographic light camera: eye = centre + direction * distance,
        box [-1, 1]^3, the caller's viewport (shadow.py:84-103)."""
        d = _arr(light_direction, np.float32)
        c = _arr(centre, np.float32)
        eye = c + d * np.float32(distance)
        view = Camera.view_matrix(eye=eye, centre=c, up=_arr(up, np.float32))
        return Camera.create(
            view=view,
            projection=Camera.orthographic_projection_matrix(-1.0, 1.0, -1.0, 1.0, -1.0, 1.0),
            viewport=_arr(viewport_matrix, np.float32),
        )

    @staticmethod
    def render_shadow_map(shadow_map, verts, faces, light_direction, viewport_matrix, centre, up,
                          strength, offset: float = 0.001, distance: float = 10.0,
                          loop_unroll: int = 1) -> "Shadow":
        """DepthShader pass of (verts, faces) into `shadow_map`, then + offset
        on every pixel (shadow.py:49-125)."""
        camera = Shadow.light_camera(light_direction, viewport_matrix, centre, up, distance)
        w, h = int(shadow_map.shape[0]), int(shadow_map.shape[1])
        spec = _jobs.JobSpec(
            shader=_lib.SHADER_DEPTH,
            width=w,
            height=h,
            viewport=camera.viewport,
            world_to_clip=camera.world_to_clip,
            world_to_eye_norm=camera.world_to_eye_norm,
            position=_jobs._host_or_device(verts, np.float32),
            faces=_jobs._host_or_device(faces, np.int32).reshape(-1, 3),
            depth_offset=float(np.asarray(offset, dtype=np.float32)),
            apply_depth_offset=True,
        )
        z, _, _, _ = render_job(spec, shadow_map, None)
        return Shadow(shadow_map=z, strength=_arr(strength, np.float32), camera=camera)

    def get(self, position) -> torch.Tensor:
        """Shadow depth at a shadow-screen position: round half away from
        zero, negative indices wrap once, outside the map reads +inf
        (shadow.py:129-153)."""
        p = torch.as_tensor(np.asarray(position, dtype=np.float32)[..., :2])
        r = torch.sign(p) * torch.floor(torch.abs(p) + 0.5)
        idx = r.to(torch.int64)
        sm = self.shadow_map
        w, h = sm.shape[0], sm.shape[1]
        i = torch.where(idx[..., 0] < 0, idx[..., 0] + w, idx[..., 0])
        j = torch.where(idx[..., 1] < 0, idx[..., 1] + h, idx[..., 1])
        ok = (i >= 0) & (i < w) & (j >= 0) & (j < h)
        vals = sm.cpu()[i.clamp(0, w - 1), j.clamp(0, h - 1)]
        return torch.where(ok, vals, torch.full_like(vals, float("inf")))


__all__ = ["Shadow"]
