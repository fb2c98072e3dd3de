"""PhongTextureShader (renderer/shaders/phong.py:65-187)."""
from typing import Any, NamedTuple

from .. import _lib
from ..shader import Shader
from ..types import LightSource


class PhongTextureExtraInput(NamedTuple):
    position: Any  # (vertices, 3) world space
    normal: Any  # (vertices, 3) world space
    uv: Any  # (vertices, 2) texel units
    light: LightSource  # direction in eye space (headlight)
    texture: Any  # (tw, th, 3)


class PhongTextureExtraFragmentData(NamedTuple):
    normal: Any = (0.0, 0.0, 0.0)
    uv: Any = (0.0, 0.0)
    colour: Any = (0.0, 0.0, 0.0)


class PhongTextureExtraMixerOutput(NamedTuple):
    canvas: Any


class PhongTextureShader(Shader):
    """Per-pixel diffuse lighting of an eye-space normal times a nearest texel."""

    kernel_id = _lib.SHADER_PHONG
    extra_input = PhongTextureExtraInput
