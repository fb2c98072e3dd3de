"""PhongReflectionShadowTextureShader
(renderer/shaders/phong_reflection_shadow.py:35-295)."""
from typing import Any, NamedTuple

from .. import _lib
from ..shader import Shader
from ..types import LightSource


class PhongReflectionShadowTextureExtraInput(NamedTuple):
    position: Any
    normal: Any
    uv: Any
    light: LightSource
    light_dir_eye: Any
    texture_shape: Any
    texture_index: Any
    texture_offset: Any
    texture: Any
    specular_map: Any
    shadow: Any  # Shadow from the light-space depth pass
    camera: Any  # the main Camera
    ambient: Any
    diffuse: Any
    specular: Any


class PhongReflectionShadowTextureExtraFragmentData(NamedTuple):
    normal: Any = (0.0, 0.0, 0.0)
    uv: Any = (0.0, 0.0)
    texture_index: Any = 0
    shadow_coord: Any = (0.0, 0.0, 0.0, 0.0)
    colour: Any = (0.0, 0.0, 0.0)


class PhongReflectionShadowTextureExtraMixerOutput(NamedTuple):
    canvas: Any


class PhongReflectionShadowTextureShader(Shader):
    """Phong reflection model with a shadow-map lookup."""

    kernel_id = _lib.SHADER_PHONG_REFLECTION_SHADOW
    extra_input = PhongReflectionShadowTextureExtraInput
