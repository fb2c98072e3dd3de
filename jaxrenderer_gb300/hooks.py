"""Compiled `primitive_chooser` / `mix` hooks: multi-candidate transparency.

The reference lets a Shader subclass override `primitive_chooser`
(renderer/shader.py:159-251) to hand more than one primitive per pixel to
interpolation and the fragment shader, and `mix` (shader.py:339-396) to
blend the resulting fragments (README.md:86-94).  Python overrides cannot
run inside the CUDA kernels, so the overrides this implementation offers are
objects assigned in place of those methods, each selecting a kernel path:

    class Glass(PhongReflectionTextureShader):
        primitive_chooser = LayeredChooser(4)
        mix = OverMixer(opacity=0.5, background=(1.0, 1.0, 1.0))

    pipeline.render(camera, Glass, buffers, face_indices, extra)

* `LayeredChooser(L)`: the L (1..4) candidates nearest to the camera (kept,
  inside, front-facing, depth not +inf) in ascending (depth, primitive id)
  order; slots past the last candidate are not kept.
* `NearestMixer()` (the default mix): the first slot the fragment shader
  keeps: the fragment shader's discard (e.g. gouraud's negative colours)
  lets the next layer show through.
* `OverMixer(opacity, background)`: front-to-back "over" compositing of the
  kept slots, T = 1, C = 0, then per slot w = T * a, C = C + w * colour,
  T = T * (1 - a); the pixel gets C + T * background and the depth and
  primitive id of the first kept slot.  `opacity` is one number for every
  face or an array with one entry per face of `face_indices`.

A pixel with no kept slot keeps its buffer values.  Gradients: the nearest
mixer's through the primitive each pixel shows; the over mixer's through
every kept slot (weight w) and to the background; opacities get none.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _lib
from .shader import Shader


@dataclass(frozen=True)
class LayeredChooser:
    """The `layers` nearest candidates of every pixel (RastJob.layers)."""

    layers: int

    def __post_init__(self):
        if not 1 <= int(self.layers) <= _lib.MAX_LAYERS:
            raise ValueError(f"LayeredChooser takes 1..{_lib.MAX_LAYERS} layers, not {self.layers}")


@dataclass(frozen=True)
class NearestMixer:
    """The default mix: the nearest kept fragment (RAST_MIX_NEAREST)."""


@dataclass(frozen=True, eq=False)
class OverMixer:
    """Front-to-back "over" compositing of the kept layers (RAST_MIX_OVER)."""

    opacity: Any = 1.0
    background: Any = (0.0, 0.0, 0.0)


def hooks_of(shader, n_faces: int) -> dict:
    """JobSpec fields (layers, mixer, opacity, background, face_alpha) for
    the chooser / mix of `shader`; raises NotImplementedError for a Python
    override, which has no kernel path."""
    chooser = getattr(shader, "primitive_chooser", Shader.primitive_chooser)
    mixer = getattr(shader, "mix", Shader.mix)
    out = {"layers": 0, "mixer": _lib.MIX_NEAREST, "opacity": 1.0, "background": (0.0, 0.0, 0.0),
           "face_alpha": None}
    if isinstance(chooser, LayeredChooser):
        out["layers"] = int(chooser.layers)
    elif chooser is not Shader.primitive_chooser:
        raise NotImplementedError("a Python primitive_chooser has no CUDA kernel path; assign "
                                  "hooks.LayeredChooser(L) instead")
    if isinstance(mixer, OverMixer):
        if out["layers"] == 0:
            raise ValueError("OverMixer blends the slots of a LayeredChooser; assign one as primitive_chooser")
        out["mixer"] = _lib.MIX_OVER
        alpha = np.asarray(mixer.opacity, np.float32)
        if alpha.ndim == 0:
            out["opacity"] = float(alpha)
        else:
            alpha = alpha.reshape(-1)
            if alpha.shape[0] != n_faces:
                raise ValueError(f"OverMixer opacity has {alpha.shape[0]} entries for {n_faces} faces")
            out["face_alpha"] = np.ascontiguousarray(alpha)
        out["background"] = tuple(np.broadcast_to(np.asarray(mixer.background, np.float32), (3,)).tolist())
    elif not isinstance(mixer, NearestMixer) and mixer is not Shader.mix:
        raise NotImplementedError("a Python mix has no CUDA kernel path; assign hooks.NearestMixer() or "
                                  "hooks.OverMixer(...) instead")
    return out


def apply_hooks(spec, shader) -> None:
    """Set the chooser / mix fields of JobSpec `spec` from `shader`."""
    for k, v in hooks_of(shader, spec.n_faces).items():
        setattr(spec, k, v)


__all__ = ["LayeredChooser", "NearestMixer", "OverMixer", "hooks_of", "apply_hooks"]
