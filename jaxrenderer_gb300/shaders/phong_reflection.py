"""PhongReflectionTextureShader (renderer/shaders/phong_reflection.py:35-258)."""
from typing import Any, NamedTuple

from .. import _lib
from ..shader import Shader
from ..types import LightSource


class PhongReflectionTextureExtraInput(NamedTuple):
    position: Any  # (vertices, 3) world space
    normal: Any  # (vertices, 3) world space
    uv: Any  # (vertices, 2) in [0, 1) repeating
    light: LightSource
    light_dir_eye: Any  # (3,) eye space
    texture_shape: Any  # (objects, 2)
    texture_index: Any  # (vertices,)
    texture_offset: Any  # scalar: MergedModel.offset
    texture: Any  # merged diffuse map
    specular_map: Any  # merged specular map
    ambient: Any
    diffuse: Any
    specular: Any


class PhongReflectionTextureExtraFragmentData(NamedTuple):
    normal: Any = (0.0, 0.0, 0.0)
    uv: Any = (0.0, 0.0)
    texture_index: Any = 0
    colour: Any = (0.0, 0.0, 0.0)


class PhongReflectionTextureExtraMixerOutput(NamedTuple):
    canvas: Any


class PhongReflectionTextureShader(Shader):
    """Phong reflection model (ambient + diffuse + specular) with merged
    diffuse and specular maps."""

    kernel_id = _lib.SHADER_PHONG_REFLECTION
    extra_input = PhongReflectionTextureExtraInput
