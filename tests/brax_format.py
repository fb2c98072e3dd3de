"""Writes batches in the reference notebooks' pickle format (not collected):
ModelObject / Model / CameraParameters under their reference module names,
arrays reduced the way jax.Array pickles (jax._src.array._reconstruct_array).
Used to exercise brax.load_batched_inputs without JAX or the reference's
own fixture files."""
from __future__ import annotations

import collections
import io
import pickle
import sys
import types

import numpy as np

from jaxrenderer_gb300.model import Model, ModelObject
from jaxrenderer_gb300.renderer import CameraParameters


def reference_pickle(objects, camera, target) -> bytes:
    names = ["renderer", "renderer.model", "renderer.renderer", "jax", "jax._src", "jax._src.array"]
    saved = {k: sys.modules.get(k) for k in names}
    mods = {k: types.ModuleType(k) for k in names}
    RModel = collections.namedtuple("Model", Model._fields)
    RObject = collections.namedtuple("ModelObject", ModelObject._fields)
    RCamera = collections.namedtuple("CameraParameters", CameraParameters._fields)
    RModel.__module__ = RObject.__module__ = "renderer.model"
    RCamera.__module__ = "renderer.renderer"
    mods["renderer.model"].Model = RModel
    mods["renderer.model"].ModelObject = RObject
    mods["renderer.renderer"].CameraParameters = RCamera

    def _reconstruct_array(fun, args, arr_state, aval_state):  # pragma: no cover - never called here
        raise AssertionError

    _reconstruct_array.__module__ = "jax._src.array"
    _reconstruct_array.__qualname__ = "_reconstruct_array"
    mods["jax._src.array"]._reconstruct_array = _reconstruct_array

    class Pickler(pickle.Pickler):
        def reducer_override(self, obj):
            if type(obj) is np.ndarray:
                fun, args, state = obj.__reduce__()
                return _reconstruct_array, (fun, args, state, {"weak_type": False, "named_shape": {}})
            return NotImplemented

    def convert(o):
        if isinstance(o, ModelObject):
            return RObject(convert(o.model), *(np.asarray(x) for x in o[1:]))
        if isinstance(o, Model):
            return RModel(*(np.asarray(x) for x in o))
        if isinstance(o, CameraParameters):
            return RCamera(*(np.asarray(x) for x in o))
        return o

    try:
        sys.modules.update(mods)
        buf = io.BytesIO()
        Pickler(buf, protocol=4).dump(([convert(o) for o in objects], convert(camera), np.asarray(target)))
        return buf.getvalue()
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
