"""pipeline.render (renderer/pipeline.py:470-537) on the GPU.

One call renders one job: the vertex shader over every vertex of
`extra[0]`, primitive set-up of every face of `face_indices`, the per-pixel
scan over every primitive, and the chosen primitive's interpolation,
fragment shader and mixer, merged into `buffers` without a depth test.  The
input buffers are not modified: new device buffers are returned, as the
reference's functional API returns new arrays.
"""
from __future__ import annotations


import numpy as np
import torch

from . import dispatch as _dispatch
from . import jobs as _jobs
from .geometry import Camera
from .hooks import apply_hooks
from .shader import kernel_id_of
from .types import Buffers


def default_device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("jaxrenderer_gb300 renders on a CUDA GPU only; none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def _faces(face_indices):
    if isinstance(face_indices, torch.Tensor):
        return face_indices.to(torch.int32).reshape(-1, 3)
    return np.ascontiguousarray(np.asarray(face_indices, dtype=np.int32).reshape(-1, 3))


def render_job(spec: _jobs.JobSpec, zbuffer, canvas, device=None, count_ties: bool = False, form=None):
    """Render one JobSpec with the form dispatch.choose picks (`form` pins
    it); returns (zbuffer, canvas or None, prim_id, near_ties tensor or None)."""
    zs, cs, ps, ties = render_jobs([spec], [zbuffer], [canvas], device, count_ties, form)
    return zs[0], cs[0], ps[0], ties


def render_jobs(specs, zbuffers, canvases, device=None, count_ties: bool = False, form=None):
    """Render several jobs as one pass (one RastBatch); returns per-job lists
    (zbuffers, canvases or None, prim_ids) and the pass's near-tie counter."""
    device = device if device is not None else default_device()
    packed = _jobs.pack(specs, zbuffers, canvases, device, want_prim_id=True, count_ties=count_ties)
    _dispatch.run(packed, form)
    out = _jobs.unpack(packed, specs)
    return [o[0] for o in out], [o[1] for o in out], [o[2] for o in out], packed.near_ties


def render_with_ids(camera: Camera, shader, buffers: Buffers, face_indices, extra,
                    loop_unroll: int = 1, count_ties: bool = False):
    """pipeline.render that also returns the winning-primitive buffer
    ((W, H) int32, -1 where nothing was written) and the near-tie count."""
    sid = kernel_id_of(shader)
    zbuffer = buffers.zbuffer
    width, height = int(zbuffer.shape[0]), int(zbuffer.shape[1])
    spec = _jobs.job_from_extra(sid, camera, extra, width, height)
    spec.faces = _faces(face_indices)
    apply_hooks(spec, shader)
    canvas = buffers.targets[0] if len(buffers.targets) > 0 else None
    z, c, p, ties = render_job(spec, zbuffer, canvas, count_ties=count_ties)
    targets = (c,) if c is not None else ()
    return Buffers(zbuffer=z, targets=targets), p, ties


def render(camera: Camera, shader, buffers: Buffers, face_indices, extra, loop_unroll: int = 1) -> Buffers:
    """Render a scene with a built-in shader (pipeline.py:470-537), with the
    default chooser / mix or the compiled hooks of `hooks` assigned to the
    shader's `primitive_chooser` / `mix`.

    The plain or the tiled form renders it, by size (dispatch.choose):
    identical buffers either way.  `loop_unroll` is accepted for API
    compatibility; the CUDA kernels have no row loop to unroll.
    """
    return render_with_ids(camera, shader, buffers, face_indices, extra, loop_unroll)[0]


__all__ = ["render", "render_with_ids", "render_job", "render_jobs", "default_device"]
