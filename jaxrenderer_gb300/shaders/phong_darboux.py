"""PhongTextureDarbouxShader (renderer/shaders/phong_darboux.py:44-316)."""
from typing import Any, NamedTuple

from .. import _lib
from ..shader import Shader
from ..types import LightSource


class PhongTextureDarbouxExtraInput(NamedTuple):
    position: Any  # (vertices, 3) world space
    normal: Any  # (vertices, 3) world space
    uv: Any  # (vertices, 2) texel units
    light: LightSource
    texture: Any  # (tw, th, 3)
    normal_map: Any  # (tw, th, 3) in the Darboux (tangent) frame
    id_to_face: Any  # (vertices,) face of each vertex
    faces_indices: Any  # (faces, 3) vertices of each face


class PhongTextureDarbouxExtraFragmentData(NamedTuple):
    normal: Any = (0.0, 0.0, 0.0)
    uv: Any = (0.0, 0.0)
    triangle: Any = None
    triangle_uv: Any = None
    colour: Any = (0.0, 0.0, 0.0)


class PhongTextureDarbouxExtraMixerOutput(NamedTuple):
    canvas: Any


class PhongTextureDarbouxShader(Shader):
    """Phong shading with the normal read from a tangent-space normal map."""

    kernel_id = _lib.SHADER_PHONG_DARBOUX
    extra_input = PhongTextureDarbouxExtraInput
