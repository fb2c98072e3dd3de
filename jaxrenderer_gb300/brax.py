"""Batched Brax inputs, as the reference's notebooks render them.

The notebooks (`notebooks/84x84/A100.ipynb`, cells 4 and 7) load a pickle of
`(batched_instances, batched_camera, batched_target)`: a list of ModelObjects
whose every array has a leading frame axis, CameraParameters with a leading
frame axis, and the per-frame camera target; each frame is rendered with
`Renderer.get_camera_image` under Light(direction=(0.57735, -0.57735,
0.57735), ambient=0.8, diffuse=0.8, specular=0.6), Shadow(centre=target),
then clamped to [0, 1], scaled to uint8 and transposed for display.

`load_batched_inputs` reads such a pickle without JAX (a whitelisting
unpickler: only the array, ModelObject, Model and CameraParameters
reconstructors are resolved; anything else is refused), and
`scenes_from_batched` turns it into InstancedScenes (one scene per frame,
the meshes shared) plus the camera / light / shadow settings above.
`save_batched_npz` / `load_batched_npz` hold the same inputs in a
compressed NumPy archive, which loads without unpickling.
"""
from __future__ import annotations

import io
import pickle
import zipfile
from dataclasses import dataclass
from typing import List, Union

import numpy as np

from .instancing import InstancedScenes, MeshLibrary
from .model import Model, ModelObject
from .renderer import CameraParameters, LightParameters, ShadowParameters

F32 = np.float32


def _reconstruct_array(fun, args, arr_state, aval_state):
    """What jax.Array's pickle reduction calls: rebuild the NumPy value."""
    value = fun(*args)
    value.__setstate__(arr_state)
    return value


def _numpy_reconstruct():
    try:
        from numpy._core import multiarray
    except ImportError:  # NumPy < 2
        from numpy.core import multiarray
    return multiarray._reconstruct


_ALLOWED = {
    ("numpy.core.multiarray", "_reconstruct"): _numpy_reconstruct,
    ("numpy._core.multiarray", "_reconstruct"): _numpy_reconstruct,
    ("numpy", "ndarray"): lambda: np.ndarray,
    ("numpy", "dtype"): lambda: np.dtype,
    ("jax._src.array", "_reconstruct_array"): lambda: _reconstruct_array,
    ("renderer.model", "Model"): lambda: Model,
    ("renderer.model", "ModelObject"): lambda: ModelObject,
    ("renderer.renderer", "CameraParameters"): lambda: CameraParameters,
    ("renderer", "Model"): lambda: Model,
    ("renderer", "ModelObject"): lambda: ModelObject,
    ("renderer", "CameraParameters"): lambda: CameraParameters,
}


class _Unpickler(pickle.Unpickler):
    def find_class(self, module, name):
        make = _ALLOWED.get((module, name))
        if make is None:
            raise pickle.UnpicklingError(f"refusing to load {module}.{name}")
        return make()


def load_batched_inputs(source: Union[str, bytes]):
    """(batched ModelObjects, batched CameraParameters, batched target) from
    a pickle file, a zip holding `inputs.pickle`, or the pickle's bytes."""
    if isinstance(source, (bytes, bytearray)):
        data = bytes(source)
    elif str(source).endswith(".zip"):
        with zipfile.ZipFile(source) as z:
            data = z.read("inputs.pickle")
    else:
        with open(source, "rb") as fh:
            data = fh.read()
    objects, camera, target = _Unpickler(io.BytesIO(data)).load()
    return list(objects), camera, np.asarray(target, F32)


# ------------------------------------------------ pickle-free archive format

_CAMERA_FIELDS = ("viewWidth", "viewHeight", "viewDepth", "near", "far", "hfov", "vfov", "position", "target", "up")


def save_batched_npz(path, objects: List[ModelObject], camera: CameraParameters, target, source_sha256: str = ""):
    """Write batched Brax inputs (the triple load_batched_inputs returns) as
    a compressed .npz: every ModelObject array and camera field with its
    leading frame axis, except arrays equal in every frame, which are stored
    once (key suffix ".shared").  Unlike the pickle, loading it runs no code."""
    n_frames = int(np.asarray(objects[0].transform).shape[0])
    arrays = {"n_objects": np.asarray(len(objects)), "n_frames": np.asarray(n_frames),
              "target": np.asarray(target, F32), "source_sha256": np.asarray(source_sha256)}

    def put(key, value):
        a = np.asarray(value)
        if a.ndim >= 1 and a.shape[0] == n_frames and all(np.array_equal(a[0], a[f]) for f in range(1, n_frames)):
            arrays[key + ".shared"] = a[0]
        else:
            arrays[key] = a

    for i, o in enumerate(objects):
        for field in Model._fields:
            put(f"o{i}.model.{field}", getattr(o.model, field))
        for field in ("local_scaling", "transform", "double_sided"):
            put(f"o{i}.{field}", getattr(o, field))
    for field in _CAMERA_FIELDS:
        arrays[f"camera.{field}"] = np.asarray(getattr(camera, field))
    np.savez_compressed(path, **arrays)


def load_batched_npz(path):
    """(batched ModelObjects, batched CameraParameters, batched target) from
    an archive written by save_batched_npz; arrays stored once are broadcast
    back to their frame axis (read-only views)."""
    with np.load(path, allow_pickle=False) as z:
        n_objects, n_frames = int(z["n_objects"]), int(z["n_frames"])

        def get(key):
            if key in z.files:
                return z[key]
            a = z[key + ".shared"]
            return np.broadcast_to(a, (n_frames,) + a.shape)

        objects = []
        for i in range(n_objects):
            model = Model(*(get(f"o{i}.model.{field}") for field in Model._fields))
            objects.append(ModelObject(model=model, local_scaling=get(f"o{i}.local_scaling"),
                                       transform=get(f"o{i}.transform"), double_sided=get(f"o{i}.double_sided")))
        camera = CameraParameters(**{field: z[f"camera.{field}"] for field in _CAMERA_FIELDS})
        return objects, camera, np.asarray(z["target"], F32)


@dataclass
class BraxBatch:
    scenes: InstancedScenes
    camera: CameraParameters  # shared fields; positions / targets per scene in `scenes`
    light: LightParameters
    shadow: ShadowParameters  # centre (frames, 3)


def _frame(a, f):
    return np.asarray(a)[f]


def _pad(m: np.ndarray, shape) -> np.ndarray:
    return np.pad(m, [(0, shape[i] - m.shape[i]) for i in range(len(shape))] + [(0, 0)] * (m.ndim - len(shape)))


def scenes_from_batched(objects: List[ModelObject], camera: CameraParameters, target, frames=None,
                        repeat: int = 1) -> BraxBatch:
    """One scene per frame (frames `frames`, all by default, the list
    repeated `repeat` times to make larger batches).  Meshes must be the
    same in every frame (only transforms and cameras move)."""
    n_frames = int(np.asarray(objects[0].transform).shape[0])
    frames = list(range(n_frames)) if frames is None else list(frames)
    frames = frames * repeat
    models, mesh_of = [], []
    keys = {}
    for o in objects:
        m = o.model
        geo = tuple(np.asarray(getattr(m, k)) for k in ("verts", "norms", "uvs", "faces", "faces_norm", "faces_uv"))
        for g in geo:
            if not all(np.array_equal(g[0], g[f]) for f in range(1, n_frames)):
                raise ValueError("mesh geometry changes between frames; only transforms may move")
        key = b"".join(g[0].tobytes() for g in geo)
        if key not in keys:
            keys[key] = len(models)
            models.append(Model(*(g[0] for g in geo), np.zeros((1, 1, 3), F32), np.zeros((1, 1), F32)))
        mesh_of.append(keys[key])
    O = len(objects)
    dshape = [np.asarray(o.model.diffuse_map).shape[1:3] for o in objects]
    T = max(max(w, h) for w, h in dshape)
    sshape = [np.asarray(o.model.specular_map).shape[1:3] for o in objects]
    if len(set(sshape)) != 1 or sshape[0][0] != sshape[0][1]:
        raise ValueError("specular maps of one batch must share one square shape")
    Ts = sshape[0][0]
    S = len(frames)
    I = S * O
    transforms = np.empty((I, 4, 4), F32)
    scaling = np.empty((I, 3), F32)
    diffuse = np.zeros((I, T, T, 3), F32)
    specular = np.empty((I, Ts, Ts), F32)
    shapes = np.empty((I, 2), np.int32)
    for si, f in enumerate(frames):
        for oi, o in enumerate(objects):
            i = si * O + oi
            transforms[i] = _frame(o.transform, f)
            scaling[i] = _frame(o.local_scaling, f)
            d = _frame(o.model.diffuse_map, f)
            diffuse[i, : d.shape[0], : d.shape[1]] = d
            shapes[i] = d.shape[:2]
            specular[i] = _frame(o.model.specular_map, f)
    cam_frames = np.asarray(frames)
    inst = InstancedScenes(MeshLibrary.from_models(models), np.tile(np.asarray(mesh_of, np.int32), S),
                           np.arange(S + 1, dtype=np.int64) * O, transforms, scaling, diffuse, specular,
                           np.asarray(camera.position, F32)[cam_frames], np.asarray(camera.target, F32)[cam_frames],
                           shapes)

    def one(x):
        a = np.asarray(x)
        if a.ndim >= 1 and a.shape[0] == n_frames:
            if not all(np.array_equal(a[0], a[f]) for f in range(n_frames)):
                raise ValueError("camera parameters other than position / target must not change per frame")
            a = a[0]
        return a.item() if a.ndim == 0 else a

    cam = CameraParameters(viewWidth=int(one(camera.viewWidth)), viewHeight=int(one(camera.viewHeight)),
                           viewDepth=float(one(camera.viewDepth)), near=float(one(camera.near)),
                           far=float(one(camera.far)), hfov=float(one(camera.hfov)), vfov=float(one(camera.vfov)),
                           position=inst.camera_position[0], target=inst.camera_target[0],
                           up=np.asarray(one(camera.up), F32))
    light = LightParameters(direction=np.array((0.57735, -0.57735, 0.57735), F32), ambient=np.full(3, 0.8, F32),
                            diffuse=np.full(3, 0.8, F32), specular=np.full(3, 0.6, F32))
    shadow = ShadowParameters(centre=np.asarray(target, F32)[cam_frames])
    return BraxBatch(inst, cam, light, shadow)


def scene_batch(bb: BraxBatch, width: int, height: int, device=None):
    """SceneBatch + DeviceMerge of a BraxBatch rendered into width x height
    canvases as Renderer.get_camera_image does: the camera's own viewport,
    a shadow map of the canvas size seen through that viewport."""
    from .batch import scene_batch_from_instances

    return scene_batch_from_instances(bb.scenes, width, height, bb.light, bb.shadow, (width, height), device,
                                      bb.camera, shadow_viewport="camera")


__all__ = ["load_batched_inputs", "save_batched_npz", "load_batched_npz", "scenes_from_batched", "scene_batch",
           "BraxBatch"]
