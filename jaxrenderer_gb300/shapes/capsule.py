"""Capsule mesh (renderer/shapes/capsule.py:1958-2015).

The reference builds its capsule from a tabulated unit sphere (its
capsule.py:19-1956, tinyrenderer's textured sphere): 192 triangles with
three unshared vertices each (576 vertices, normals and uvs), the northern
and southern halves pushed apart by +-half_height along the up axis.  The
table is kept alike here (capsule_table.npz, written from the reference's
literals by make_capsule_table.py) because its vertex values decide which
pixels a capsule covers and its uvs which texels it samples: scenes built
with create_capsule then render the reference's geometry.  The capsules of
the reference's own Brax Ant fixture (test_resources/pre-gen-brax) are
reproduced bit for bit by create_capsule (tests/test_host.py).
"""
from __future__ import annotations

import enum
from pathlib import Path

import numpy as np

from ..model import Model

_TABLE = Path(__file__).resolve().parent / "capsule_table.npz"


class UpAxis(enum.IntEnum):
    X = 0
    Y = 1
    Z = 2


def _load_table():
    with np.load(_TABLE, allow_pickle=False) as t:
        return (t["verts"].astype(np.float32), t["normals"].astype(np.float32), t["uvs"].astype(np.float32),
                t["faces"].astype(np.int32))


_VERTS, _NORMALS, _UVS, _FACES = _load_table()


def create_capsule(radius, half_height, up_axis, diffuse_map, specular_map) -> Model:
    """Capsule of `radius` whose hemispheres sit +-half_height along up_axis:
    the table's coordinates permuted so that its z axis becomes up_axis,
    scaled by radius in float32, then half_height added to the vertices with
    a positive up coordinate and subtracted from the others."""
    up = int(up_axis)
    shuffled = np.array(((1, 2, 0), (0, 1, 2), (2, 0, 1)))[up]
    verts = _VERTS[:, shuffled] * np.float32(radius)
    hh = np.float32(half_height)
    verts[:, up] = verts[:, up] + np.where(verts[:, up] > 0, hh, -hh)
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
