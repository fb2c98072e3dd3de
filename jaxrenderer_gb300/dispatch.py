"""Form selection behind the reference-facing API (Renderer.render,
Renderer.get_camera_image, pipeline.render, Shadow.render_shadow_map).

Both forms give identical buffers: the plain form (the reference's own
per-pixel scan over every primitive) and the tiled form (binned tiles).
The plain form needs fewer launches, so it wins on small passes; the tiled
form's work grows with the pixels each primitive covers instead of
W * H * F, so it wins on large ones.  "auto" takes the tiled form for a pass
whose jobs test at least TILED_MIN_PAIRS pixel-triangle pairs in total, with
the autotuner's tile shape and bin capacity for the pass; the form can be
pinned with set_render_form("plain" | "tiled").
"""
from __future__ import annotations

import threading
from typing import Optional

import numpy as np
import torch

from . import _lib
from . import jobs as _jobs

FORMS = ("auto", "plain", "tiled")
# ~1e8 pixel-triangle pairs: about where the plain scan's time (at ~1.3e12
# pairs/s on a GB300) passes the tiled form's fixed launch cost
TILED_MIN_PAIRS = 1 << 27
# the tiled form's per-face pixel rectangles are 16-bit
TILED_MAX_SIDE = 65535
_state = threading.local()


def set_render_form(form: str) -> None:
    """Pin the form of this thread's renders ("auto" restores the choice by size)."""
    if form not in FORMS:
        raise ValueError(f"form must be one of {FORMS}")
    _state.form = form


def render_form() -> str:
    return getattr(_state, "form", "auto")


def pass_pairs(packed: _jobs.PackedBatch) -> int:
    """Pixel-triangle pairs the plain form tests for this pass: sum of W * H * F."""
    return sum(int(j.width) * int(j.height) * int(j.n_faces) for j in packed.jobs)


def choose(packed: _jobs.PackedBatch, form: Optional[str] = None) -> str:
    f = form or render_form()
    if f == "auto":
        if any(int(j.width) > TILED_MAX_SIDE or int(j.height) > TILED_MAX_SIDE for j in packed.jobs):
            return "plain"
        return "tiled" if pass_pairs(packed) >= TILED_MIN_PAIRS else "plain"
    if f not in ("plain", "tiled"):
        raise ValueError(f"form must be one of {FORMS}")
    return f


def job_array(packed: _jobs.PackedBatch) -> np.ndarray:
    """The batch's job table as a structured array with the RastJob layout."""
    return np.frombuffer(bytes(packed.jobs), dtype=np.dtype(_lib.RastJob)).copy()


def tuned_config(packed: _jobs.PackedBatch) -> "_lib.RastTiledConfig":
    """The autotuner's RastTiledConfig for this pass (cached per workload
    class).  When it has to time candidates it renders into scratch copies of
    the outputs, so the caller's buffers see one render only."""
    from .autotune import tiled_config_for_batch

    b = _lib.RastBatch.from_buffer_copy(packed.batch)
    scratch = []

    def alias(name, t):
        if t is not None:
            c = t.clone()
            scratch.append(c)
            setattr(b.pools, name, c.data_ptr())

    alias("zbuffer", packed.zbuffer)
    alias("canvas", packed.canvas)
    alias("prim_id", packed.prim_id)
    alias("layer_prim", packed.layer_prim)
    b.near_ties = None
    cfg = tiled_config_for_batch(packed.zbuffer.device, b, job_array(packed))
    del scratch
    return cfg


def run(packed: _jobs.PackedBatch, form: Optional[str] = None, stream: Optional[torch.cuda.Stream] = None) -> str:
    """Render a packed pass with the chosen form (stream-ordered); returns it."""
    f = choose(packed, form)
    if f == "plain":
        _jobs.render_plain(packed, stream)
    else:
        _jobs.render_tiled_config(packed, tuned_config(packed), stream)
    return f


__all__ = ["FORMS", "TILED_MIN_PAIRS", "set_render_form", "render_form", "choose", "run", "tuned_config",
           "pass_pairs"]
