"""The seven built-in shaders of jaxrenderer, each a CUDA kernel path."""
from .depth import DepthExtraInput, DepthShader
from .gouraud import GouraudExtraInput, GouraudShader
from .gouraud_texture import GouraudTextureExtraInput, GouraudTextureShader
from .phong import PhongTextureExtraInput, PhongTextureShader
from .phong_darboux import PhongTextureDarbouxExtraInput, PhongTextureDarbouxShader
from .phong_reflection import PhongReflectionTextureExtraInput, PhongReflectionTextureShader
from .phong_reflection_shadow import (
    PhongReflectionShadowTextureExtraInput,
    PhongReflectionShadowTextureShader,
)

__all__ = [
    "DepthExtraInput",
    "DepthShader",
    "GouraudExtraInput",
    "GouraudShader",
    "GouraudTextureExtraInput",
    "GouraudTextureShader",
    "PhongTextureExtraInput",
    "PhongTextureShader",
    "PhongTextureDarbouxExtraInput",
    "PhongTextureDarbouxShader",
    "PhongReflectionTextureExtraInput",
    "PhongReflectionTextureShader",
    "PhongReflectionShadowTextureExtraInput",
    "PhongReflectionShadowTextureShader",
]
