"""jaxrenderer_gb300: jaxrenderer's rasterisation path on one GB300 GPU.

Drop-in for the reference's public names (renderer/__init__.py of
JoeyTeng/jaxrenderer): `Renderer.get_camera_image`, `pipeline.render`
(exported as `render`), the built-in shaders, `Model`/`ModelObject`/
`merge_objects`, `Camera`, `CameraParameters`, `LightParameters`,
`ShadowParameters`.  Host set-up runs in NumPy; every per-vertex,
per-primitive and per-pixel stage runs in hand-written sm_103a CUDA kernels
reached through the C ABI in include/rast_gb300.h.
"""
from typing import Dict as DictT
from typing import List, NamedTuple, ParamSpec, Sequence, Tuple, Type, TypeAlias

from . import hooks, shaders
from .batch import SceneBatch, render_batch
from .geometry import Camera, normalise, quaternion, quaternion_mul, rotation_matrix
from .hooks import LayeredChooser, NearestMixer, OverMixer
from .model import Model, ModelObject, batch_models, merge_objects
from .pipeline import render, render_with_ids
from .renderer import CameraParameters, LightParameters, Renderer, ShadowParameters
from .shader import Shader
from .shadow import Shadow
from .shapes import UpAxis, create_capsule, create_cube
from .types import Buffers, Colour, JaxFloating, JaxInteger, LightSource, SpecularMap, Texture, Vec3f
from .utils import build_texture_from_PyTinyrenderer, transpose_for_display


def add_tracing_name(func):
    """Named-scope decorator of the reference (_meta_utils.py:16-31); the
    CUDA path carries no trace annotations, so this returns `func`."""
    return func


def jit(func=None, **_kwargs):
    """The reference's typed_jit (_meta_utils.py:58-78).  Nothing here is
    traced or compiled at call time, so this returns `func`."""
    if func is None:
        return lambda f: f
    return func


def replace_dict(d, **kwargs):
    out = dict(d)
    out.update(kwargs)
    return out


__all__ = [
    "add_tracing_name",
    "batch_models",
    "Buffers",
    "build_texture_from_PyTinyrenderer",
    "Camera",
    "CameraParameters",
    "Colour",
    "create_capsule",
    "create_cube",
    "DictT",
    "JaxFloating",
    "JaxInteger",
    "jit",
    "LayeredChooser",
    "LightParameters",
    "LightSource",
    "List",
    "merge_objects",
    "Model",
    "ModelObject",
    "NamedTuple",
    "NearestMixer",
    "normalise",
    "OverMixer",
    "ParamSpec",
    "quaternion_mul",
    "quaternion",
    "render",
    "render_batch",
    "render_with_ids",
    "Renderer",
    "replace_dict",
    "rotation_matrix",
    "SceneBatch",
    "Sequence",
    "Shader",
    "Shadow",
    "ShadowParameters",
    "SpecularMap",
    "Texture",
    "transpose_for_display",
    "Tuple",
    "Type",
    "TypeAlias",
    "UpAxis",
    "Vec3f",
    "shaders",
]
