"""Differentiable rendering: a torch.autograd.Function over the CUDA forward
and the hand-written backward (rast_backward), plus torch versions of the
camera construction so gradients reach camera positions and light
directions (renderer.py:141-196, geometry.py:536-684 of the reference).

    db = DifferentiableBatch(scene_batch)
    canvas, zbuffer = db.render(position=pos, texture=tex,
                                world_to_clip=w2c, world_to_eye_norm=w2e,
                                light_direction=ldir)
    loss(canvas).backward()

Visibility is piecewise constant: gradients flow through the winning
primitive of every pixel, as under jax.grad of the reference.  A
DifferentiableBatch keeps one forward state: call backward before the next
render.
"""
from __future__ import annotations

from typing import Tuple

import numpy as np
import torch

from . import _lib
from .batch import BatchRunner, SceneBatch

PARAM_COLUMNS = {
    "world_to_clip": (_lib.GRAD_WORLD_TO_CLIP, 16),
    "world_to_eye_norm": (_lib.GRAD_WORLD_TO_EYE_NORM, 16),
    "light_direction": (_lib.GRAD_LIGHT_DIRECTION, 3),
    "light_colour": (_lib.GRAD_LIGHT_COLOUR, 3),
    "light_dir_eye": (_lib.GRAD_LIGHT_DIR_EYE, 3),
    "ambient": (_lib.GRAD_AMBIENT, 3),
    "diffuse": (_lib.GRAD_DIFFUSE, 3),
    "specular": (_lib.GRAD_SPECULAR, 3),
    "shadow_strength": (_lib.GRAD_SHADOW_STRENGTH, 3),
    "background": (_lib.GRAD_BACKGROUND, 3),
}
POOL_PARAMS = ("position", "normal", "colour", "texture", "specular_map", "normal_map")
JOB_OFFSETS = {name: getattr(_lib.RastJob, name).offset // 4 for name in PARAM_COLUMNS}


# ------------------------------------------------------ torch camera math

def _normalise(v: torch.Tensor) -> torch.Tensor:
    return v / torch.sqrt((v[..., 0:1] * v[..., 0:1] + v[..., 1:2] * v[..., 1:2]) + v[..., 2:3] * v[..., 2:3])


def view_matrix(eye: torch.Tensor, centre: torch.Tensor, up: torch.Tensor) -> torch.Tensor:
    """lookAt (geometry.py:536-575), batched over leading axes."""
    forward = _normalise(centre - eye)
    up = _normalise(up.expand_as(forward))
    side = _normalise(torch.cross(forward, up, dim=-1))
    up = torch.cross(side, forward, dim=-1)
    zero = torch.zeros_like(eye[..., :1])
    one = torch.ones_like(zero)
    r0 = torch.cat([side, -(side * eye).sum(-1, keepdim=True)], -1)
    r1 = torch.cat([up, -(up * eye).sum(-1, keepdim=True)], -1)
    r2 = torch.cat([-forward, (forward * eye).sum(-1, keepdim=True)], -1)
    r3 = torch.cat([zero, zero, zero, one], -1)
    return torch.stack([r0, r1, r2, r3], dim=-2)


def view_matrix_inv(eye: torch.Tensor, centre: torch.Tensor, up: torch.Tensor) -> torch.Tensor:
    """Inverse of lookAt from its parts (geometry.py:581-632)."""
    forward = _normalise(centre - eye)
    up = _normalise(up.expand_as(forward))
    side = _normalise(torch.cross(forward, up, dim=-1))
    up = torch.cross(side, forward, dim=-1)
    rot = torch.stack([side, up, -forward], dim=-1)  # columns
    top = torch.cat([rot, eye.unsqueeze(-1)], -1)
    zero = torch.zeros_like(top[..., :1, :3])
    bottom = torch.cat([zero, torch.ones_like(zero[..., :1])], -1)  # (0, 0, 0, 1), no host copy
    return torch.cat([top, bottom], dim=-2)


def perspective_projection_matrix(fovy: float, aspect: float, z_near: float, z_far: float, dtype=torch.float32,
                                  device=None) -> torch.Tensor:
    """gluPerspective (geometry.py:638-684)."""
    f = float(1.0 / np.tan(np.radians(fovy) / 2.0))
    p = torch.zeros((4, 4), dtype=dtype, device=device)
    p[0, 0] = float(f / aspect)
    p[1, 1] = f
    p[2, 2] = float((z_far + z_near) / (z_near - z_far))
    p[2, 3] = float(2.0 * z_far * z_near / (z_near - z_far))
    p[3, 2] = -1.0
    return p


def camera_matrices(eye: torch.Tensor, params, target=None, up=None) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    """(world_to_clip, world_to_eye_norm, view) of cameras at `eye` (N, 3)
    built as Renderer.create_camera_from_parameters does.  With `target` and
    `up` given as tensors on eye's device, calls after the first for the same
    camera parameters copy nothing from the host, so they can be captured in
    a CUDA graph."""
    dt, dev = eye.dtype, eye.device

    def vec(x, default):
        if isinstance(x, torch.Tensor):
            return x.to(dtype=dt, device=dev)
        return torch.as_tensor(np.asarray(default if x is None else x, np.float64), dtype=dt, device=dev)

    target = vec(target, params.target)
    up = vec(up, params.up)
    target = target.expand_as(eye)
    v = view_matrix(eye, target, up)
    vinv = view_matrix_inv(eye, target, up)
    aspect = np.tan(np.radians(params.hfov) / 2.0) / np.tan(np.radians(params.vfov) / 2.0)
    key = (float(params.vfov), float(aspect), float(params.near), float(params.far), dt, dev)
    p = _PROJECTIONS.get(key)
    if p is None:  # built once per camera and device: later calls copy nothing from the host
        p = perspective_projection_matrix(params.vfov, aspect, params.near, params.far, dtype=dt, device=dev)
        _PROJECTIONS[key] = p
    return p @ v, vinv.transpose(-1, -2), v


_PROJECTIONS: dict = {}


def apply_vec(vec: torch.Tensor, m: torch.Tensor) -> torch.Tensor:
    """Camera.apply_vec (geometry.py:352-389) of one vector by (N, 4, 4) matrices."""
    n = _normalise(vec)
    h = torch.cat([n, torch.zeros_like(n[..., :1])], -1)
    t = (m @ h.unsqueeze(-1)).squeeze(-1)[..., :3]
    return _normalise(t)


# ------------------------------------------------------------ the Function

class _RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, db: "DifferentiableBatch", names: Tuple[str, ...], *tensors):
        runner = db.runner
        jf = runner.job_floats()
        for name, t in zip(names, tensors):
            if name in POOL_PARAMS:
                runner.pools[name].copy_(t.detach().reshape(runner.pools[name].shape))
            else:
                off = JOB_OFFSETS[name]
                width = PARAM_COLUMNS[name][1]
                jf[:, off : off + width] = t.detach().reshape(jf.shape[0], width).to(torch.float32)
        out = runner.run()
        ctx.db = db
        ctx.names = names
        ctx.shapes = [t.shape for t in tensors]
        ctx.dtypes = [t.dtype for t in tensors]
        db._generation += 1
        ctx.generation = db._generation
        return out.canvas.clone(), out.zbuffer.clone()

    @staticmethod
    def backward(ctx, g_canvas, g_zbuffer):
        db = ctx.db
        if db._generation != ctx.generation:
            raise RuntimeError("DifferentiableBatch was re-rendered before backward of an earlier render")
        g = db.runner.backward(g_canvas, g_zbuffer)
        grads = []
        for name, shape, dt in zip(ctx.names, ctx.shapes, ctx.dtypes):
            if name in POOL_PARAMS:
                grads.append(g[name].reshape(shape).to(dt))
            else:
                col, width = PARAM_COLUMNS[name]
                grads.append(g["job_params"][:, col : col + width].reshape(shape).to(dt))
        return (None, None, *grads)


class DifferentiableBatch:
    """Differentiable renders of one SceneBatch (main pass gradients)."""

    def __init__(self, sb: SceneBatch, form: str = "tiled", tiled_config=None):
        self.runner = BatchRunner(sb, form=form, want_prim_id=True, tiled_config=tiled_config)
        self._generation = 0

    def render(self, **params: torch.Tensor):
        """Render with the given tensors in place of the batch's inputs.

        Pool inputs: position, normal, colour (gouraud), texture,
        specular_map, normal_map (flat pool shapes).  Per-scene inputs, (N, ...): world_to_clip (N, 4, 4),
        world_to_eye_norm (N, 4, 4), light_direction, light_colour,
        light_dir_eye, ambient, diffuse, specular, shadow_strength (N, 3).
        Returns (canvas (N, W, H, 3), zbuffer (N, W, H))."""
        for k in params:
            if k not in POOL_PARAMS and k not in PARAM_COLUMNS:
                raise KeyError(f"unknown differentiable input {k!r}")
        names = tuple(params)
        return _RenderFunction.apply(self, names, *[params[k] for k in names])


__all__ = ["DifferentiableBatch", "camera_matrices", "view_matrix", "view_matrix_inv",
           "perspective_projection_matrix", "apply_vec"]
