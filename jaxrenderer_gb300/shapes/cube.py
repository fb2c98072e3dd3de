"""Axis-aligned box with a texture atlas (renderer/shapes/cube.py:144-159).

24 vertices (4 per side, each side with its own normal and uv patch) and 12
triangles.  The vertex order, winding and atlas layout are the reference's
(they define which texel every pixel samples); they are generated here from a
per-side description instead of a literal table.
"""
from __future__ import annotations

import numpy as np

from ..model import Model

# Per side: (normal, the four corners as sign triples, atlas uv of each
# corner in quarters, the two triangles in corner indices 0..3).
_SIDES = (
    ((0, 0, 1), ((-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)), ((3, 1), (4, 1), (4, 0), (3, 0)), ((0, 1, 2), (0, 2, 3))),
    ((0, 0, -1), ((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1)), ((2, 1), (1, 1), (1, 0), (2, 0)), ((2, 1, 0), (3, 2, 0))),
    ((-1, 0, 0), ((-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1)), ((2, 0), (3, 0), (3, 1), (2, 1)), ((2, 1, 0), (3, 2, 0))),
    ((1, 0, 0), ((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)), ((1, 2), (1, 1), (0, 1), (0, 2)), ((0, 1, 2), (0, 2, 3))),
    ((0, -1, 0), ((-1, -1, -1), (-1, -1, 1), (1, -1, 1), (1, -1, -1)), ((1, 2), (1, 1), (2, 1), (2, 2)), ((2, 1, 0), (3, 2, 0))),
    ((0, 1, 0), ((-1, 1, -1), (-1, 1, 1), (1, 1, 1), (1, 1, -1)), ((0, 0), (0, 1), (1, 1), (1, 0)), ((0, 1, 2), (0, 2, 3))),
)


def _tables():
    verts, norms, uvs, faces = [], [], [], []
    for s, (normal, corners, uv4, tris) in enumerate(_SIDES):
        for c, q in zip(corners, uv4):
            verts.append(c)
            norms.append(normal)
            uvs.append((q[0] / 4.0, q[1] / 4.0))
        faces.extend(tuple(4 * s + k for k in t) for t in tris)
    return (
        np.asarray(verts, dtype=np.float32),
        np.asarray(norms, dtype=np.float32),
        np.asarray(uvs, dtype=np.float32),
        np.asarray(faces, dtype=np.int32),
    )


_VERTS, _NORMALS, _UVS, _FACES = _tables()


def create_cube(half_extents, texture_scaling, diffuse_map, specular_map) -> Model:
    """Box of the given half extents; uv scaled by texture_scaling."""
    he = np.asarray(half_extents, dtype=np.float32)
    ts = np.asarray(texture_scaling, dtype=np.float32)
    return Model(
        verts=_VERTS * he,
        norms=_NORMALS.copy(),
        uvs=_UVS * ts,
        faces=_FACES.copy(),
        faces_norm=_FACES.copy(),
        faces_uv=_FACES.copy(),
        diffuse_map=np.asarray(diffuse_map, dtype=np.float32),
        specular_map=np.asarray(specular_map, dtype=np.float32),
    )
