"""GouraudTextureShader (renderer/shaders/gouraud_texture.py:55-167)."""
from typing import Any, NamedTuple

from .. import _lib
from ..shader import Shader
from ..types import LightSource


class GouraudTextureExtraInput(NamedTuple):
    position: Any  # (vertices, 3) world space
    normal: Any  # (vertices, 3) world space
    uv: Any  # (vertices, 2) texel units
    light: LightSource
    texture: Any  # (tw, th, 3)


class GouraudTextureExtraFragmentData(NamedTuple):
    colour: Any = (0.0, 0.0, 0.0)
    uv: Any = (0.0, 0.0)


class GouraudTextureExtraMixerOutput(NamedTuple):
    canvas: Any


class GouraudTextureShader(Shader):
    """Per-vertex light colour times a nearest texel (uv in texel units,
    wrapped by the texture size)."""

    kernel_id = _lib.SHADER_GOURAUD_TEXTURE
    extra_input = GouraudTextureExtraInput
