"""Instanced scenes: meshes uploaded once, objects placed per frame.

The reference merges a scene's ModelObjects on the host inside every traced
render call (`merge_objects`, renderer/model.py:447-555) and then gathers
positions, normals, uvs and texture indices per face corner
(renderer/renderer.py:277-295).  Here a batch of scenes is described once as
a mesh library plus, per scene, a run of instances (mesh id, per-instance
texture maps); per frame only the instances' transforms and local scalings
change, and `rast_merge_objects` rebuilds the per-corner pools on the device
with the same operations as the host `merge_objects` + `flatten_corners`
(checked bit for bit by the tests).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from .model import Model, ModelObject, merge_objects

F32 = np.float32
MESH_DTYPE = np.dtype(_lib.RastMesh)
INSTANCE_DTYPE = np.dtype(_lib.RastInstance)


@dataclass
class MeshLibrary:
    """Concatenated geometry of the meshes instances refer to."""

    models: List[Model]
    verts: np.ndarray
    norms: np.ndarray
    uvs: np.ndarray
    faces: np.ndarray
    faces_norm: np.ndarray
    faces_uv: np.ndarray
    table: np.ndarray  # MESH_DTYPE per mesh

    @classmethod
    def from_models(cls, models: Sequence[Model]) -> "MeshLibrary":
        models = list(models)
        table = np.zeros(len(models), MESH_DTYPE)
        parts = {k: [] for k in ("verts", "norms", "uvs", "faces", "faces_norm", "faces_uv")}
        rows = {"verts": 0, "norms": 0, "uvs": 0, "faces": 0}
        for i, m in enumerate(models):
            v, n, u = (np.asarray(m.verts, F32).reshape(-1, 3), np.asarray(m.norms, F32).reshape(-1, 3),
                       np.asarray(m.uvs, F32).reshape(-1, 2))
            f, fn, fu = (np.asarray(x, np.int32).reshape(-1, 3) for x in (m.faces, m.faces_norm, m.faces_uv))
            if not (len(f) == len(fn) == len(fu)):
                raise ValueError(f"mesh {i}: faces, faces_norm and faces_uv differ in length")
            table[i] = (rows["verts"], rows["norms"], rows["uvs"], rows["faces"], len(v), len(n), len(u), len(f))
            for k, a in (("verts", v), ("norms", n), ("uvs", u), ("faces", f), ("faces_norm", fn), ("faces_uv", fu)):
                parts[k].append(a)
            rows["verts"] += len(v)
            rows["norms"] += len(n)
            rows["uvs"] += len(u)
            rows["faces"] += len(f)
        cat = {k: np.concatenate(p, axis=0) if p else np.zeros((0, 2 if k == "uvs" else 3),
                                                                np.int32 if k.startswith("faces") else F32)
               for k, p in parts.items()}
        return cls(models, cat["verts"], cat["norms"], cat["uvs"], cat["faces"], cat["faces_norm"],
                   cat["faces_uv"], table)


@dataclass
class InstancedScenes:
    """Scenes of instances.  Scene s owns instances [scene_begin[s],
    scene_begin[s + 1]); instance i draws mesh `mesh[i]` with ModelObject
    `transform[i]` / `local_scaling[i]` and its own T x T diffuse and
    specular maps (merged per scene as merge_maps does: concatenated)."""

    library: MeshLibrary
    mesh: np.ndarray  # (I,) int32
    scene_begin: np.ndarray  # (S + 1,) int64
    transforms: np.ndarray  # (I, 4, 4) float32
    local_scaling: np.ndarray  # (I, 3) float32
    diffuse: np.ndarray  # (I, T, T, 3) float32, zero-padded at the end of each axis
    specular: np.ndarray  # (I, Ts, Ts) float32
    camera_position: np.ndarray  # (S, 3)
    camera_target: Optional[np.ndarray] = None
    texture_shape: Optional[np.ndarray] = None  # (I, 2) the diffuse maps' own sizes; (T, T) when None

    @property
    def n_scenes(self) -> int:
        return len(self.scene_begin) - 1

    @property
    def n_instances(self) -> int:
        return len(self.mesh)

    @property
    def tex_size(self) -> int:
        return int(self.diffuse.shape[1])

    @property
    def spec_size(self) -> int:
        return int(self.specular.shape[1])

    def shapes(self) -> np.ndarray:
        if self.texture_shape is not None:
            return np.asarray(self.texture_shape, np.int32).reshape(-1, 2)
        return np.tile(np.array([[self.tex_size] * 2], np.int32), (self.n_instances, 1))

    def check_maps(self) -> None:
        """merge_maps pads a scene's maps to the scene's largest; the batch
        layout pads to the batch's, so every scene must hold a map of the
        batch's (T, T) size (as with a textured ground in every scene)."""
        sh = self.shapes()
        T = self.tex_size
        for s in range(self.n_scenes):
            a, b = int(self.scene_begin[s]), int(self.scene_begin[s + 1])
            if b > a and (sh[a:b, 0].max() != T or sh[a:b, 1].max() != T):
                raise ValueError(f"scene {s}: its largest diffuse map is not {T}x{T}")

    def subset(self, begin: int, end: int) -> "InstancedScenes":
        """Scenes [begin, end) as their own batch (the mesh library shared)."""
        i0, i1 = int(self.scene_begin[begin]), int(self.scene_begin[end])
        cut = lambda a: None if a is None else a[begin:end]  # noqa: E731
        return InstancedScenes(self.library, self.mesh[i0:i1], self.scene_begin[begin : end + 1] - i0,
                               self.transforms[i0:i1], self.local_scaling[i0:i1], self.diffuse[i0:i1],
                               self.specular[i0:i1], self.camera_position[begin:end], cut(self.camera_target),
                               None if self.texture_shape is None else self.texture_shape[i0:i1])

    def _mesh_counts(self, field: str) -> np.ndarray:
        return self.library.table[field][self.mesh].astype(np.int64)

    @property
    def n_faces(self) -> np.ndarray:
        """Triangles per scene."""
        return np.add.reduceat(self._mesh_counts("n_faces"), self.scene_begin[:-1]).astype(np.int32) \
            if self.n_instances else np.zeros(self.n_scenes, np.int32)

    def instance_table(self) -> np.ndarray:
        """RastInstance rows (static: everything but the transforms)."""
        t = np.zeros(self.n_instances, INSTANCE_DTYPE)
        scene_of = np.repeat(np.arange(self.n_scenes), np.diff(self.scene_begin))
        first = self.scene_begin[scene_of]
        t["mesh"] = self.mesh
        t["scene_first"] = first
        t["scene_count"] = np.diff(self.scene_begin)[scene_of]
        for field, off, tot, row in (("n_verts", "vert_offset", "scene_verts", "vert_row"),
                                     ("n_norms", "norm_offset", "scene_norms", "norm_row"),
                                     ("n_uvs", "uv_offset", "scene_uvs", "uv_row")):
            c = self._mesh_counts(field)
            incl = np.cumsum(c)
            t[row] = incl - c
            start_of_scene = np.concatenate([[0], incl])[self.scene_begin[:-1]]
            t[off] = (incl - c) - start_of_scene[scene_of]
            t[tot] = (np.concatenate([[0], incl])[self.scene_begin[1:]] - start_of_scene)[scene_of]
        corners = 3 * self._mesh_counts("n_faces")
        t["corner_begin"] = np.cumsum(corners) - corners
        return t

    def corner_begin(self) -> np.ndarray:
        """First per-corner row of every scene."""
        corners = 3 * self._mesh_counts("n_faces")
        cb = np.concatenate([[0], np.cumsum(corners)])
        return cb[self.scene_begin[:-1]].astype(np.int64)

    def objects(self, s: int) -> List[ModelObject]:
        """Scene s as the reference's ModelObjects (per-instance maps)."""
        out = []
        for i in range(int(self.scene_begin[s]), int(self.scene_begin[s + 1])):
            m = self.library.models[int(self.mesh[i])]
            w, h = (int(x) for x in self.shapes()[i])
            model = m._replace(diffuse_map=self.diffuse[i][:w, :h], specular_map=self.specular[i])
            out.append(ModelObject(model=model, local_scaling=self.local_scaling[i], transform=self.transforms[i]))
        return out

    def shell(self):
        """A FlatScenes with the batch's bookkeeping and no per-corner arrays."""
        from .synthetic import FlatScenes

        self.check_maps()
        T = self.tex_size
        counts = np.diff(self.scene_begin)
        return FlatScenes(None, None, None, None, self.diffuse.reshape(-1, T, 3),
                          self.specular.reshape(-1, self.spec_size), self.corner_begin(), self.n_faces,
                          (T * self.scene_begin[:-1]).astype(np.int64), counts.astype(np.int32),
                          np.asarray(self.camera_position, F32), T,
                          None if self.camera_target is None else np.asarray(self.camera_target, F32),
                          self.shapes(), self.spec_size)

    def host_flat(self, scenes: Sequence[int]):
        """FlatScenes of `scenes` built by the host reference path:
        merge_objects + Renderer.flatten_corners per scene."""
        from .renderer import Renderer
        from .synthetic import FlatScenes

        T = self.tex_size
        pos, nrm, uv, tix, tex, spec, nf, no = [], [], [], [], [], [], [], []
        for s in scenes:
            merged = merge_objects(self.objects(int(s)))
            p, n, u, t, _ = Renderer.flatten_corners(merged)
            pos.append(p), nrm.append(n), uv.append(u), tix.append(t)
            tex.append(np.asarray(merged.diffuse_map, F32).reshape(-1, T, 3))
            spec.append(np.asarray(merged.specular_map, F32).reshape(-1, self.spec_size))
            nf.append(len(p) // 3)
            no.append(int(self.scene_begin[s + 1] - self.scene_begin[s]))
        nf = np.asarray(nf, np.int32)
        no = np.asarray(no, np.int32)
        sel = np.asarray(scenes, np.int64)
        shapes = np.concatenate([self.shapes()[int(self.scene_begin[s]):int(self.scene_begin[s + 1])] for s in scenes])
        return FlatScenes(np.concatenate(pos), np.concatenate(nrm), np.concatenate(uv),
                          np.concatenate(tix).astype(np.int32), np.concatenate(tex), np.concatenate(spec),
                          np.concatenate([[0], np.cumsum(3 * nf.astype(np.int64))[:-1]]), nf,
                          np.concatenate([[0], np.cumsum(T * no.astype(np.int64))[:-1]]), no,
                          np.asarray(self.camera_position, F32)[sel], T,
                          None if self.camera_target is None else np.asarray(self.camera_target, F32)[sel],
                          shapes, self.spec_size)


class DeviceMerge:
    """Device-resident mesh library + instance table of an InstancedScenes;
    `merge()` rebuilds the per-corner pools with rast_merge_objects."""

    def __init__(self, inst: InstancedScenes, pools, device=None):
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        lib = inst.library
        T = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a)).to(device=dev, dtype=dt)  # noqa: E731
        self.inst = inst
        self.device = dev
        self.lib = _lib.load()
        self.t = {
            "meshes": torch.from_numpy(lib.table.view(np.uint8).copy()).to(dev),
            "instances": torch.from_numpy(inst.instance_table().view(np.uint8).copy()).to(dev),
            "verts": T(lib.verts), "norms": T(lib.norms), "uvs": T(lib.uvs),
            "faces": T(lib.faces, torch.int32), "faces_norm": T(lib.faces_norm, torch.int32),
            "faces_uv": T(lib.faces_uv, torch.int32),
        }
        self.transforms = T(inst.transforms.reshape(-1, 16))
        self.local_scaling = T(inst.local_scaling.reshape(-1, 3))
        self.pools = pools
        b = _lib.RastMergeBatch()
        b.meshes = self.t["meshes"].data_ptr()
        b.n_meshes = len(lib.table)
        b.n_instances = inst.n_instances
        b.instances = self.t["instances"].data_ptr()
        b.transforms = self.transforms.data_ptr()
        b.local_scaling = self.local_scaling.data_ptr()
        for name, key in (("mesh_verts", "verts"), ("mesh_norms", "norms"), ("mesh_uvs", "uvs"),
                          ("mesh_faces", "faces"), ("mesh_faces_norm", "faces_norm"), ("mesh_faces_uv", "faces_uv")):
            setattr(b, name, self.t[key].data_ptr())
        b.total_faces = int(inst._mesh_counts("n_faces").sum())
        b.total_verts = int(inst._mesh_counts("n_verts").sum())
        b.total_norms = int(inst._mesh_counts("n_norms").sum())
        b.total_uvs = int(inst._mesh_counts("n_uvs").sum())
        for name in ("position", "normal", "uv", "texture_index"):
            t = pools.get(name)
            setattr(b, name, t.data_ptr() if t is not None else None)
        self.batch = b
        nbytes = int(self.lib.rast_merge_workspace_bytes(ctypes.byref(b)))
        self.ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev)
        self.ws_bytes = nbytes

    def merge(self, transforms=None, local_scaling=None, stream: Optional[torch.cuda.Stream] = None) -> None:
        """Optionally copy new transforms (I, 4, 4) / local scalings (I, 3)
        (host or device tensors; pinned host memory copies asynchronously),
        then rebuild the per-corner pools on `stream`."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        with torch.cuda.stream(s):
            if transforms is not None:
                self.transforms.copy_(torch.as_tensor(transforms).reshape(-1, 16), non_blocking=True)
            if local_scaling is not None:
                self.local_scaling.copy_(torch.as_tensor(local_scaling).reshape(-1, 3), non_blocking=True)
        _lib.check(self.lib.rast_merge_objects(ctypes.byref(self.batch), self.ws.data_ptr(), self.ws_bytes,
                                               s.cuda_stream), "rast_merge_objects")


def instanced_pools(inst: InstancedScenes, device) -> dict:
    """Device pools of an instanced batch: per-corner arrays allocated (the
    merge fills them), faces 3 * arange, merged texture and specular maps."""
    corners = int(3 * inst.n_faces.astype(np.int64).sum())
    max_f = int(inst.n_faces.max()) if inst.n_scenes else 0
    T = inst.tex_size
    return {
        "position": torch.empty((corners, 3), dtype=torch.float32, device=device),
        "normal": torch.empty((corners, 3), dtype=torch.float32, device=device),
        "uv": torch.empty((corners, 2), dtype=torch.float32, device=device),
        "texture_index": torch.empty(corners, dtype=torch.int32, device=device),
        "faces": torch.arange(3 * max_f, dtype=torch.int32, device=device).reshape(-1, 3),
        "texture": torch.as_tensor(inst.diffuse.reshape(-1, T, 3)).to(device),
        "specular_map": torch.as_tensor(inst.specular.reshape(-1, inst.spec_size)).to(device),
        "texture_shape": torch.as_tensor(inst.shapes()).to(device),
    }


__all__ = ["MeshLibrary", "InstancedScenes", "DeviceMerge", "instanced_pools", "MESH_DTYPE", "INSTANCE_DTYPE"]
