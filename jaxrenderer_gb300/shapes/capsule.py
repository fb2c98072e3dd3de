"""Capsule mesh (renderer/shapes/capsule.py:1958-2015).

A unit sphere of 12 longitude segments x 9 latitude bands (20 degrees each),
split at the equator, the two halves pushed apart by +-half_height along the
up axis: 192 triangles with 3 vertices each (576 vertices, no sharing), the
reference's tessellation.  The reference takes its vertex values from a
tabulated sphere; this one is generated, so coordinates differ in the last
digits while counts, winding, normal directions and uv layout agree.
"""
from __future__ import annotations

import enum

import numpy as np

from ..model import Model


class UpAxis(enum.IntEnum):
    X = 0
    Y = 1
    Z = 2


_SEGMENTS = 12
_BANDS = 9


def _sphere():
    verts, norms, uvs = [], [], []

    def point(band_edge: int, seg: int):
        theta = np.pi * band_edge / _BANDS  # polar angle from +z
        phi = 2.0 * np.pi * seg / _SEGMENTS
        n = (np.sin(theta) * np.sin(phi), np.sin(theta) * np.cos(phi), np.cos(theta))
        uv = (seg / _SEGMENTS, 1.0 - band_edge / _BANDS)
        return n, uv

    def tri(*pts):
        for b, s in pts:
            n, uv = point(b, s)
            verts.append(n)
            norms.append(n)
            uvs.append(uv)

    for b in range(_BANDS):
        for s in range(_SEGMENTS):
            a00, a01, a10, a11 = (b, s), (b, s + 1), (b + 1, s), (b + 1, s + 1)
            # counter-clockwise seen from outside
            if b == 0:  # north cap: one triangle per segment
                tri(a00, a11, a10)
            elif b == _BANDS - 1:  # south cap
                tri(a00, a01, a10)
            else:
                tri(a00, a11, a10)
                tri(a00, a01, a11)
    v = np.asarray(verts, dtype=np.float32)
    return v, np.asarray(norms, dtype=np.float32), np.asarray(uvs, dtype=np.float32)


_VERTS, _NORMALS, _UVS = _sphere()
_FACES = np.arange(len(_VERTS), dtype=np.int32).reshape(-1, 3)


def create_capsule(radius, half_height, up_axis, diffuse_map, specular_map) -> Model:
    """Capsule of `radius` whose hemispheres sit +-half_height along up_axis."""
    up = int(up_axis)
    shuffled = np.array(((1, 2, 0), (0, 1, 2), (2, 0, 1)))[up]
    verts = _VERTS[:, shuffled] * np.float32(radius)
    verts[:, up] = verts[:, up] + np.where(verts[:, up] > 0, np.float32(half_height), -np.float32(half_height))
    return Model(
        verts=verts.astype(np.float32),
        norms=_NORMALS[:, shuffled].copy(),
        uvs=_UVS.copy(),
        faces=_FACES.copy(),
        faces_norm=_FACES.copy(),
        faces_uv=_FACES.copy(),
        diffuse_map=np.asarray(diffuse_map, dtype=np.float32),
        specular_map=np.asarray(specular_map, dtype=np.float32),
    )
