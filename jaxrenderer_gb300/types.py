"""Data types of the rasteriser's public API (renderer/types.py of jaxrenderer).

Arrays are x-major as in the reference: a canvas is (width, height, channel)
and a z-buffer (width, height).  Host inputs are NumPy arrays (or anything
`numpy.asarray` accepts); buffers produced by the CUDA path are torch tensors
on the GPU.
"""
from __future__ import annotations

from typing import Any, NamedTuple, Tuple, TypeVar

import numpy as np

# Shape-documenting aliases (types.py:63-155).
Canvas = Any  # (width, height, channel)
ZBuffer = Any  # (width, height)
Colour = Any  # (channel,)
Vec2i = Any
Vec3i = Any
Vec2f = Any
Vec3f = Any
Vec4f = Any
Triangle = Any  # (3, 4)
FaceIndices = Any  # (faces, 3)
Vertices = Any  # (vertices, 3)
Normals = Any  # (normals, 3)
UVCoordinates = Any  # (uv_counts, 2)
Texture = Any  # (textureWidth, textureHeight, channel)
SpecularMap = Any  # (textureWidth, textureHeight)
NormalMap = Any  # (textureWidth, textureHeight, 3)
CanvasMask = Any
BoolV = Any
FloatV = Any
IntV = Any
NumV = Any
JaxFloating = np.floating
JaxInteger = np.integer


class DtypeInfo(NamedTuple):
    """finfo / iinfo summary (types.py:95-131)."""

    min: Any
    max: Any
    bits: int
    dtype: Any

    @classmethod
    def create(cls, dtype) -> "DtypeInfo":
        dt = np.dtype(dtype)
        if np.issubdtype(dt, np.floating):
            fi = np.finfo(dt)
            return cls(min=dt.type(fi.min), max=dt.type(fi.max), bits=fi.bits, dtype=dt.type)
        if np.issubdtype(dt, np.integer):
            ii = np.iinfo(dt)
            return cls(min=ii.min, max=ii.max, bits=ii.bits, dtype=dt.type)
        raise ValueError(f"Unexpected dtype {dtype}")


class LightSource(NamedTuple):
    """Parallel light (types.py:134-145)."""

    direction: Any = np.array((0.0, 0.0, -1.0), dtype=np.float32)
    """in world space, as it goes from that position to origin (camera)."""
    colour: Any = np.ones(3, dtype=np.float32)


_TargetsT = TypeVar("_TargetsT")


class Buffers(NamedTuple):
    """z-buffer plus extra target buffers (types.py:148-155)."""

    zbuffer: Any
    targets: Tuple[Any, ...]


__all__ = [
    "Buffers",
    "Canvas",
    "Colour",
    "DtypeInfo",
    "LightSource",
    "SpecularMap",
    "Texture",
    "Vec3f",
    "ZBuffer",
]
