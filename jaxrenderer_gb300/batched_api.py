"""Renderer.get_camera_image over a leading batch axis: the reference's
notebooks call jax.jit(jax.vmap(Renderer.get_camera_image)) on ModelObjects,
CameraParameters and shadow centres that carry one leading axis of frames
(notebooks/84x84/A100.ipynb cells 4-7, examples/batch_rendering.py:87-95).

All frames render as one batch per pass.  When the frames share their
meshes and maps (only transforms, local scalings, camera positions /
targets and shadow centres change from frame to frame, as in the Brax
batches) and the light is one for all frames, the batch is instanced:
meshes and maps are uploaded once, and every call copies the frames'
transforms and scalings to the device, rebuilds the per-corner pools there
(rast_merge_objects, bit for bit the host merge_objects), refreshes the
job tables with the frames' camera and light-space matrices (vectorised,
bit for bit the per-frame set-up) and renders both passes in the form
dispatch picks for them.  That set-up is kept between calls, keyed by the
identity and shape of the mesh and map arrays (as jax.jit keys its traces
by shapes): arrays already seen are not read again, so mutate none of them
in place between calls.  Any other batch (meshes or maps that change
between frames, one light or Camera matrix set per frame) merges every
frame on the host and renders through Renderer.render's batched path.
"""
from __future__ import annotations

from collections import OrderedDict
from typing import Optional

import numpy as np
import torch

from . import dispatch
from .batch import BatchRunner, frame_matrices, scene_batch_from_instances, scene_batch_tables
from .instancing import InstancedScenes, MeshLibrary
from .model import Model, merge_objects
from .pipeline import default_device
from .renderer import CameraParameters, Renderer

F32 = np.float32
MAX_CACHED = 4
_CACHE: "OrderedDict[tuple, _Prepared]" = OrderedDict()

_MESH = ("verts", "norms", "uvs", "faces", "faces_norm", "faces_uv")
_MAPS = ("diffuse_map", "specular_map")
_RANK = Renderer._UNBATCHED_NDIM["Model"]


def _frames(a, rank: int, B: int) -> np.ndarray:
    """`a` with its frame axis (a read-only broadcast when it has none)."""
    a = np.asarray(a)
    return a if a.ndim == rank + 1 else np.broadcast_to(a, (B,) + a.shape)


def _first(a, rank: int) -> np.ndarray:
    a = np.asarray(a)
    return a[0] if a.ndim == rank + 1 else a


def _same_every_frame(a, rank: int) -> bool:
    a = np.asarray(a)
    return a.ndim == rank or bool(np.array_equal(a, np.broadcast_to(a[:1], a.shape)))


class _Prepared:
    """Instanced set-up of one batch structure: library, pools, device
    merge and a BatchRunner, reused by every call with the same structure."""

    def __init__(self, inst: InstancedScenes, objects, params: CameraParameters, light, shadow_param,
                 width: int, height: int, device, form: str):
        self.inst = inst
        self.refs = [getattr(o.model, f) for o in objects for f in _MESH + _MAPS]  # keep identities valid
        self.params = params
        self.width, self.height = width, height
        self.shadow = shadow_param is not None
        self.sb, self.merge = scene_batch_from_instances(inst, width, height, light, shadow_param, (width, height),
                                                         device, params, shadow_viewport="camera")
        self.form = form
        self.runner = BatchRunner(self.sb, form=form, want_prim_id=False)
        self.tables = None  # job tables of the last call, and the light / shadow set-up they hold
        self.setup_key = None


def _setup_key(light, shadow_param, params) -> bytes:
    """Everything in the job tables besides the per-frame matrices."""
    parts = [np.asarray(x, F32).tobytes() for x in light]
    if shadow_param is not None:
        parts += [np.asarray(shadow_param.up, F32).tobytes(), np.asarray(shadow_param.strength, F32).tobytes(),
                  np.asarray(shadow_param.offset, F32).tobytes(), bytes([np.ndim(shadow_param.centre)])]
    parts += [repr(tuple(getattr(params, f) for f in ("viewWidth", "viewHeight", "viewDepth", "near", "far", "hfov",
                                                      "vfov"))).encode(), np.asarray(params.up, F32).tobytes()]
    return b"|".join(parts)


def _structure_key(objects, B, width, height, shadow, form, device):
    ids = tuple((id(getattr(o.model, f)), np.shape(getattr(o.model, f))) for o in objects for f in _MESH + _MAPS)
    return (B, int(width), int(height), bool(shadow), form, str(device), ids)


def _instanced(objects, B: int, positions: np.ndarray, targets: np.ndarray) -> Optional[InstancedScenes]:
    """InstancedScenes of B frames of `objects`, or None when meshes or maps
    change between frames or the maps do not merge into one square map
    (merge_maps pads a scene's maps to its widest and tallest; the instanced
    layout pads to a square)."""
    models, mesh_of, keys = [], [], {}
    for o in objects:
        m = o.model
        if not all(_same_every_frame(getattr(m, f), _RANK[f]) for f in _MESH + _MAPS):
            return None
        geo = tuple(np.ascontiguousarray(_first(getattr(m, f), _RANK[f])) for f in _MESH)
        key = b"".join(g.tobytes() + str(g.shape).encode() for g in geo)
        if key not in keys:
            keys[key] = len(models)
            models.append(Model(*geo, np.zeros((1, 1, 3), F32), np.zeros((1, 1), F32)))
        mesh_of.append(keys[key])
    dmaps = [np.asarray(_first(o.model.diffuse_map, 3), F32) for o in objects]
    smaps = [np.asarray(_first(o.model.specular_map, 2), F32) for o in objects]
    if any(d.ndim != 3 or d.shape[2] != 3 for d in dmaps):
        return None
    T = max(d.shape[0] for d in dmaps)
    if max(d.shape[1] for d in dmaps) != T:
        return None
    if len({s.shape for s in smaps}) != 1 or smaps[0].shape[0] != smaps[0].shape[1]:
        return None
    O = len(objects)
    diffuse = np.zeros((O, T, T, 3), F32)
    for k, d in enumerate(dmaps):
        diffuse[k, : d.shape[0], : d.shape[1]] = d
    shapes = np.asarray([d.shape[:2] for d in dmaps], np.int32)
    transforms, scaling = _placements(objects, B)
    return InstancedScenes(MeshLibrary.from_models(models), np.tile(np.asarray(mesh_of, np.int32), B),
                           np.arange(B + 1, dtype=np.int64) * O, transforms, scaling,
                           np.broadcast_to(diffuse, (B,) + diffuse.shape).reshape((B * O,) + diffuse.shape[1:]),
                           np.broadcast_to(np.stack(smaps), (B, O) + smaps[0].shape).reshape((B * O,) + smaps[0].shape),
                           positions, targets, np.tile(shapes, (B, 1)))


def _placements(objects, B: int):
    """(B * O, 4, 4) transforms and (B * O, 3) local scalings, frame-major."""
    tr = np.stack([_frames(o.transform, 2, B) for o in objects], axis=1).astype(F32, copy=False)
    sc = np.stack([_frames(o.local_scaling, 1, B) for o in objects], axis=1).astype(F32, copy=False)
    return np.ascontiguousarray(tr.reshape(-1, 4, 4)), np.ascontiguousarray(sc.reshape(-1, 3))


def _shared_params(camera: CameraParameters, B: int):
    """(CameraParameters of the shared fields, positions (B, 3), targets (B, 3)),
    or None when a field other than position / target changes per frame."""
    ranks = Renderer._UNBATCHED_NDIM["CameraParameters"]
    shared = {}
    for name in camera._fields:
        v = getattr(camera, name)
        if name in ("position", "target"):
            continue
        if np.ndim(v) == ranks[name] + 1:
            if not _same_every_frame(v, ranks[name]):
                return None
            v = np.asarray(v)[0]
        shared[name] = v.item() if np.ndim(v) == 0 and hasattr(v, "item") else v
    pos = np.ascontiguousarray(_frames(np.asarray(camera.position, F32), 1, B))
    tgt = np.ascontiguousarray(_frames(np.asarray(camera.target, F32), 1, B))
    params = CameraParameters(**shared, position=pos[0], target=tgt[0])
    return params, pos, tgt


def _light_is_shared(light) -> bool:
    return Renderer._batch_size(light) is None


def _shadow_is_fast(shadow_param) -> bool:
    if shadow_param is None:
        return True
    ranks = Renderer._UNBATCHED_NDIM["ShadowParameters"]
    return all(np.ndim(getattr(shadow_param, f)) == ranks[f] for f in ("up", "strength", "offset"))


def get_camera_image(objects, light, camera, width: int, height: int, colour_default, zbuffer_default,
                     shadow_param, B: int) -> torch.Tensor:
    """(B, width, height, 3) canvases of B frames (see the module docstring)."""
    device = default_device()
    if isinstance(camera, CameraParameters) and _light_is_shared(light) and _shadow_is_fast(shadow_param):
        shared = _shared_params(camera, B)
        if shared is not None:
            params, pos, tgt = shared
            out = _render_instanced(objects, light, params, pos, tgt, width, height, colour_default,
                                    zbuffer_default, shadow_param, B, device)
            if out is not None:
                return out
    return _render_per_frame(objects, light, camera, width, height, colour_default, zbuffer_default, shadow_param,
                             B, device)


def _render_instanced(objects, light, params, pos, tgt, width, height, colour_default, zbuffer_default,
                      shadow_param, B, device) -> Optional[torch.Tensor]:
    form = dispatch.render_form()
    key = _structure_key(objects, B, width, height, shadow_param is not None, form, device)
    prep = _CACHE.get(key)
    if prep is None:
        inst = _instanced(objects, B, pos, tgt)
        if inst is None:
            return None
        if form == "auto":  # the pass sizes decide; both forms give the same canvases
            pairs = int(width) * int(height) * int(inst.n_faces.astype(np.int64).sum())
            form = "tiled" if pairs * (2 if shadow_param is not None else 1) >= dispatch.TILED_MIN_PAIRS else "plain"
        prep = _Prepared(inst, objects, params, light, shadow_param, width, height, device, form)
        _CACHE[key] = prep
        while len(_CACHE) > MAX_CACHED:
            _CACHE.popitem(last=False)
    else:
        _CACHE.move_to_end(key)
        inst = prep.inst
        inst.transforms, inst.local_scaling = _placements(objects, B)
        inst.camera_position, inst.camera_target = pos, tgt
        prep.merge.merge(inst.transforms, inst.local_scaling)
    if shadow_param is not None and np.ndim(shadow_param.centre) == 1:
        shadow_param = shadow_param._replace(centre=np.broadcast_to(np.asarray(shadow_param.centre, F32), (B, 3)))
    skey = _setup_key(light, shadow_param, params)
    if prep.tables is None or prep.setup_key != skey:
        prep.tables = scene_batch_tables(inst.shell(), width, height, light, shadow_param, (width, height), params,
                                         shadow_viewport="camera")
        prep.setup_key = skey
    else:  # same light and shadow set-up: only the frames' matrices change
        frame_matrices(prep.tables, pos, tgt, params, light, shadow_param)
    t = prep.tables
    r = prep.runner
    r.set_job_tables(t.main_jobs, t.shadow_jobs)
    r.set_colour_default(colour_default)
    r.run(zbuffer_default=float(np.asarray(zbuffer_default, F32)))
    return r.canvas.clone()


def _render_per_frame(objects, light, camera, width, height, colour_default, zbuffer_default, shadow_param, B,
                      device) -> torch.Tensor:
    scenes = []
    for b in range(B):
        cam = Renderer._take(camera, b)
        cam = Renderer.create_camera_from_parameters(cam) if isinstance(cam, CameraParameters) else cam
        model = merge_objects(Renderer._take(list(objects), b))
        scenes.append((model, Renderer._take(light, b), cam, Renderer._take(shadow_param, b)))
    buffers = Renderer.create_buffers(width, height, B, colour_default, zbuffer_default, device)
    zbs = [buffers.zbuffer[b] for b in range(B)]
    cvs = [buffers.targets[0][b] for b in range(B)]
    _, canvases, _ = Renderer._render_scenes(scenes, zbs, cvs, device)
    return torch.stack(canvases)


__all__ = ["get_camera_image", "MAX_CACHED"]
