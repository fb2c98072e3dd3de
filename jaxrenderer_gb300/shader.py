"""Shader interface (renderer/shader.py of jaxrenderer).

The reference runs user-defined Python shaders inside its JAX program.  Here
the seven built-in shaders (renderer/shaders/*.py) are CUDA kernel paths,
selected by class exactly as the reference selects its static shader class;
a `Shader` subclass without a kernel raises NotImplementedError when it is
rendered.  The stage methods of this base class describe the contract each
kernel path implements; calling them from Python is not supported (there is
no CPU fallback).
"""
from __future__ import annotations

from typing import Any, NamedTuple, Optional


class PerVertex(NamedTuple):
    """Built-in output of the vertex shader (shader.py:42-51)."""

    gl_Position: Any


class PerFragment(NamedTuple):
    """Built-in output of the fragment shader (shader.py:54-64)."""

    gl_FragDepth: Any = float("inf")
    keeps: Any = True
    use_default_depth: Any = False


class MixerOutput(NamedTuple):
    """Built-in output of Shader.mix (shader.py:80-88)."""

    keep: Any
    zbuffer: Any


class Shader:
    """Base class of shaders (shader.py:91).

    `kernel_id` names the CUDA kernel path (RastShader in rast_gb300.h) of a
    built-in shader; it is None for user-defined shaders, which this
    implementation cannot run.
    """

    kernel_id: Optional[int] = None
    extra_input: Any = None  # the shader's ExtraInput NamedTuple class

    @staticmethod
    def vertex(gl_VertexID, gl_InstanceID, camera, extra):
        """Vertex stage (shader.py:103-153): gl_Position + varyings."""
        raise NotImplementedError("shader stages run inside the CUDA kernels only")

    @staticmethod
    def primitive_chooser(gl_FragCoord, gl_FrontFacing, gl_PointCoord, keeps, values,
                          barycentric_screen, barycentric_clip):
        """Default: nearest kept front-facing primitive, first index on ties
        (shader.py:159-251)."""
        raise NotImplementedError("shader stages run inside the CUDA kernels only")

    @staticmethod
    def interpolate(values, barycentric_screen, barycentric_clip):
        """Default: perspective-correct (SMOOTH) interpolation (shader.py:257-290)."""
        raise NotImplementedError("shader stages run inside the CUDA kernels only")

    @staticmethod
    def fragment(gl_FragCoord, gl_FrontFacing, gl_PointCoord, varying, extra):
        """Default: keep, default depth (shader.py:296-333)."""
        raise NotImplementedError("shader stages run inside the CUDA kernels only")

    @staticmethod
    def mix(gl_FragDepth, keeps, extra):
        """Default: nearest kept fragment (shader.py:339-396)."""
        raise NotImplementedError("shader stages run inside the CUDA kernels only")


def kernel_id_of(shader) -> int:
    kid = getattr(shader, "kernel_id", None)
    if kid is None:
        raise NotImplementedError(
            f"{getattr(shader, '__name__', shader)!r} has no CUDA kernel path: only the built-in "
            "shaders (DepthShader, GouraudShader, GouraudTextureShader, PhongTextureShader, "
            "PhongTextureDarbouxShader, PhongReflectionTextureShader, "
            "PhongReflectionShadowTextureShader) can be rendered"
        )
    return int(kid)


ID = int

__all__ = ["PerVertex", "PerFragment", "MixerOutput", "Shader", "kernel_id_of", "ID"]
