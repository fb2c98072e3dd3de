"""Meshes and their merge into one scene (renderer/model.py of jaxrenderer).

`merge_objects` applies each object's local scaling and model matrix to its
vertices and the inverse-transpose to its normals, concatenates faces with
index offsets, and pads + concatenates the texture maps along axis 0
(model.py:447-555).  It runs on the host in NumPy, in FP32 with the
reference's operation order.
"""
from __future__ import annotations

from typing import Any, List, NamedTuple, Sequence, Tuple

import numpy as np

from .geometry import Camera, _arr, lu_inverse, transform_matrix_from_rotation


class Model(NamedTuple):
    """Mesh with attached maps (model.py:37-143)."""

    verts: Any
    norms: Any
    uvs: Any
    faces: Any
    faces_norm: Any
    faces_uv: Any
    diffuse_map: Any
    specular_map: Any

    @classmethod
    def create(cls, verts, norms, uvs, faces, diffuse_map, specular_map=None) -> "Model":
        """faces_norm and faces_uv default to faces; specular map to 2.0."""
        diffuse_map = _arr(diffuse_map)
        if specular_map is None:
            specular_map = np.full(diffuse_map.shape[:2], 2.0, dtype=np.float32)
        faces = np.asarray(faces, dtype=np.int32)
        return cls(
            verts=_arr(verts),
            norms=_arr(norms),
            uvs=_arr(uvs),
            faces=faces,
            faces_norm=faces,
            faces_uv=faces,
            diffuse_map=diffuse_map,
            specular_map=_arr(specular_map),
        )

    def value_checks(self) -> List[str]:
        """Index range checks (model.py:105-143); returns the problems found."""
        errors = []
        for name, idx, n in (
            ("faces", self.faces, len(self.verts)),
            ("faces_norm", self.faces_norm, len(self.norms)),
            ("faces_uv", self.faces_uv, len(self.uvs)),
        ):
            idx = np.asarray(idx)
            if idx.size and (idx.min() < 0 or idx.max() >= n):
                errors.append(f"{name} out of bound, expected [0, {n}), got {idx.max()}.")
        return errors


class MergedModel(NamedTuple):
    """All objects of a scene merged into one mesh (model.py:155-339)."""

    verts: Any
    norms: Any
    uvs: Any
    faces: Any
    faces_norm: Any
    faces_uv: Any
    texture_index: Any
    double_sided: Any
    texture_shape: Any
    offset: int
    diffuse_map: Any
    specular_map: Any

    @staticmethod
    def generate_object_vert_info(counts: Sequence[int], values: Sequence[Any]) -> np.ndarray:
        parts = [np.full((c,) + np.asarray(v).shape, v) for c, v in zip(counts, values)]
        return np.concatenate(parts, axis=0)

    @staticmethod
    def merge_verts(vs: Sequence[np.ndarray], fs: Sequence[np.ndarray]) -> Tuple[np.ndarray, np.ndarray]:
        cumsum = np.concatenate([[0], np.cumsum([len(v) for v in vs[:-1]])]).astype(np.int32)
        dtype = np.result_type(*vs)
        verts = np.concatenate([np.asarray(v).astype(dtype) for v in vs], axis=0)
        faces = np.concatenate([np.asarray(f, dtype=np.int32) + cumsum[i] for i, f in enumerate(fs)], axis=0)
        return verts, faces

    @staticmethod
    def merge_maps(maps: Sequence[np.ndarray]) -> Tuple[np.ndarray, Tuple[int, int]]:
        """Pad every map to the largest shape (zeros at the end of each axis)
        and concatenate along axis 0 (model.py:249-301)."""
        maps = [np.asarray(m) for m in maps]
        dims = maps[0].ndim
        single = tuple(max(m.shape[i] for m in maps) for i in range(dims))
        dtype = np.result_type(*maps)
        padded = [
            np.pad(m, [(0, single[i] - m.shape[i]) for i in range(dims)]).astype(dtype)
            for m in maps
        ]
        return np.concatenate(padded, axis=0), (single[0], single[1])

    @staticmethod
    def uv_repeat(uv, shape, map_index, offset) -> np.ndarray:
        """Tile-repeat uv into the merged map (model.py:306-339)."""
        uv = _arr(uv)
        whole = np.where(uv >= 0, np.floor(uv), np.ceil(uv))
        frac = uv - whole
        frac = np.where(frac < 0, frac + np.asarray(1, dtype=uv.dtype), frac)
        out = frac * np.asarray(shape).astype(uv.dtype)
        out[..., 0] = out[..., 0] + np.asarray(np.asarray(map_index) * np.asarray(offset)).astype(uv.dtype)
        return out


class ModelObject(NamedTuple):
    """A model placed in the world (model.py:342-421)."""

    model: Model
    local_scaling: Any = np.ones(3, dtype=np.float32)
    transform: Any = np.identity(4, dtype=np.float32)
    double_sided: Any = False

    def replace_with_position(self, position) -> "ModelObject":
        t = np.array(_arr(self.transform), copy=True)
        t[:3, 3] = _arr(position)
        return self._replace(transform=t)

    def replace_with_orientation(self, orientation=None, rotation_matrix=None) -> "ModelObject":
        if rotation_matrix is None:
            if orientation is None:
                orientation = np.array((0.0, 0.0, 0.0, 1.0), dtype=np.float32)
            rotation_matrix = transform_matrix_from_rotation(orientation)
        t = np.array(_arr(self.transform), copy=True)
        t[:3, :3] = _arr(rotation_matrix)
        return self._replace(transform=t)

    def replace_with_local_scaling(self, local_scaling) -> "ModelObject":
        return self._replace(local_scaling=_arr(local_scaling))

    def replace_with_double_sided(self, double_sided) -> "ModelObject":
        return self._replace(double_sided=double_sided)


def batch_models(models: Sequence[MergedModel]) -> MergedModel:
    """Stack every field on a new leading batch axis (model.py:425-442)."""
    return MergedModel._make(
        np.stack([np.asarray(m[i]) for m in models], axis=0) for i in range(len(models[0]))
    )


def merge_objects(objects: Sequence[ModelObject]) -> MergedModel:
    """Merge objects into a single model (model.py:447-555)."""
    models = [obj.model for obj in objects]
    counts = [len(m.verts) for m in models]
    map_indices = MergedModel.generate_object_vert_info(counts, list(range(len(models)))).astype(np.int32)
    map_wh = np.asarray([np.asarray(m.diffuse_map).shape[:2] for m in models], dtype=np.int32)
    double_sided = MergedModel.generate_object_vert_info(counts, [bool(o.double_sided) for o in objects])
    diffuse_map, single_shape = MergedModel.merge_maps([m.diffuse_map for m in models])
    specular_map = MergedModel.merge_maps([m.specular_map for m in models])[0]

    def transform_vert(verts, local_scaling, transform):
        return Camera.apply_pos(_arr(verts) * _arr(local_scaling), _arr(transform))

    verts, faces = MergedModel.merge_verts(
        [transform_vert(o.model.verts, o.local_scaling, o.transform) for o in objects],
        [m.faces for m in models],
    )

    def transform_normals(normals, transform):
        t = _arr(transform)
        return Camera.apply_vec(_arr(normals), np.ascontiguousarray(lu_inverse(t).T))

    norms, faces_norm = MergedModel.merge_verts(
        [transform_normals(o.model.norms, o.transform) for o in objects],
        [m.faces_norm for m in models],
    )
    uvs, faces_uv = MergedModel.merge_verts([_arr(m.uvs) for m in models], [m.faces_uv for m in models])
    return MergedModel(
        verts=verts,
        norms=norms,
        uvs=uvs,
        faces=faces,
        faces_norm=faces_norm,
        faces_uv=faces_uv,
        texture_shape=map_wh,
        texture_index=map_indices,
        double_sided=double_sided,
        offset=int(single_shape[0]),
        diffuse_map=diffuse_map,
        specular_map=specular_map,
    )


__all__ = ["Model", "MergedModel", "ModelObject", "batch_models", "merge_objects"]
