"""Scene builders shared by the CPU and GPU tests (not collected)."""
from __future__ import annotations

import numpy as np

from jaxrenderer_gb300 import _lib
from jaxrenderer_gb300.geometry import Camera
from jaxrenderer_gb300.jobs import JobSpec
from jaxrenderer_gb300.synthetic import BASE_SEED, random_triangle_soup

F32 = np.float32

ALL_SHADERS = (
    _lib.SHADER_DEPTH,
    _lib.SHADER_GOURAUD,
    _lib.SHADER_GOURAUD_TEXTURE,
    _lib.SHADER_PHONG,
    _lib.SHADER_PHONG_DARBOUX,
    _lib.SHADER_PHONG_REFLECTION,
    _lib.SHADER_PHONG_REFLECTION_SHADOW,
)


def unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(F32)


def perspective_camera(W, H, eye=(0.3, -0.2, 4.0), fovy=50.0, near=0.1, far=20.0, depth=1.0):
    view = Camera.view_matrix(np.array(eye, F32), np.zeros(3, F32), np.array((0, 1, 0), F32))
    proj = Camera.perspective_projection_matrix(fovy, W / H, near, far)
    vp = Camera.viewport_matrix(np.zeros(2, np.int32), np.array((W, H)), depth)
    return Camera.create(view, proj, vp)


def random_job(shader, seed, W=48, H=40, F=60, spread=1.6, eye=(0.3, -0.2, 4.0)):
    """A random triangle soup job for `shader` with every attribute it reads."""
    rng = np.random.Generator(np.random.PCG64(BASE_SEED + seed))
    cam = perspective_camera(W, H, eye=eye)
    verts, faces = random_triangle_soup(rng, F, spread=spread)
    V = verts.shape[0]
    spec = JobSpec(shader=shader, width=W, height=H, viewport=cam.viewport,
                   world_to_clip=cam.world_to_clip, world_to_eye_norm=cam.world_to_eye_norm,
                   position=verts, faces=faces)
    spec.normal = unit(rng, V)
    spec.light_direction = unit(rng, 1)[0]
    spec.light_colour = rng.uniform(0.5, 1.0, 3).astype(F32)
    if shader == _lib.SHADER_GOURAUD:
        spec.colour = rng.uniform(-0.2, 1.0, (V, 3)).astype(F32)
    if shader in (_lib.SHADER_GOURAUD_TEXTURE, _lib.SHADER_PHONG, _lib.SHADER_PHONG_DARBOUX):
        spec.uv = rng.uniform(-10, 20, (V, 2)).astype(F32)
        spec.texture = rng.uniform(0, 1, (7, 5, 3)).astype(F32)
    if shader == _lib.SHADER_PHONG_DARBOUX:
        spec.normal_map = unit(rng, 35).reshape(7, 5, 3)
        spec.id_to_face = (np.arange(V) // 3).astype(np.int32)
        spec.darboux_faces = faces.copy()
    if shader in (_lib.SHADER_PHONG_REFLECTION, _lib.SHADER_PHONG_REFLECTION_SHADOW):
        n_obj = 3
        shapes = np.array([(4, 4), (3, 5), (6, 2)], np.int32)
        spec.texture_shape = shapes
        spec.texture_offset = 6
        spec.texture = rng.uniform(0, 1, (6 * n_obj, 5, 3)).astype(F32)
        spec.specular_map = rng.uniform(0.5, 8, (6 * n_obj, 5)).astype(F32)
        obj = rng.integers(0, n_obj, size=F)
        spec.texture_index = np.repeat(obj, 3).astype(np.int32)
        spec.uv = rng.uniform(-2, 3, (V, 2)).astype(F32)
        spec.light_dir_eye = unit(rng, 1)[0]
        spec.ambient = rng.uniform(0, 0.6, 3).astype(F32)
        spec.diffuse = rng.uniform(0, 0.6, 3).astype(F32)
        spec.specular = rng.uniform(0, 0.3, 3).astype(F32)
    if shader == _lib.SHADER_PHONG_REFLECTION_SHADOW:
        scam = Camera.create(
            Camera.view_matrix(np.array((2.0, 3.0, 5.0), F32), np.zeros(3, F32), np.array((0, 0, 1), F32)),
            Camera.orthographic_projection_matrix(-2.0, 2.0, -2.0, 2.0, -10.0, 10.0),
            Camera.viewport_matrix(np.zeros(2, np.int32), np.array((32, 24)), 1.0),
        )
        spec.shadow_map = rng.uniform(0.2, 0.8, (32, 24)).astype(F32)
        spec.shadow_viewport = scam.viewport
        spec.shadow_world_to_clip = scam.world_to_clip
        spec.shadow_strength = rng.uniform(0.2, 0.8, 3).astype(F32)
    return spec


def initial_buffers(spec, zdefault=1.0, cdefault=(1.0, 1.0, 1.0)):
    z = np.full((spec.width, spec.height), zdefault, F32)
    c = None
    if spec.shader != _lib.SHADER_DEPTH:
        c = np.broadcast_to(np.asarray(cdefault, F32), (spec.width, spec.height, 3)).copy()
    return z, c


# ---- the reference's own smoke-test scenes (tests/smoke_test.py:27-132, :135-329)

def smoke_batched_triangles_job():
    """tests/smoke_test.py:27-102: 1920x1080, 5 triangles, GouraudShader."""
    W, H = 1920, 1080
    eye = np.array((0.0, 0, 2), F32)
    cam = Camera.create(
        view=Camera.view_matrix(eye=eye, centre=np.zeros(3, F32), up=np.array((0.0, 1, 0), F32)),
        projection=Camera.perspective_projection_matrix(fovy=90.0, aspect=1.0, z_near=-1.0, z_far=1.0),
        viewport=Camera.viewport_matrix(lowerbound=np.zeros(2, np.int32), dimension=np.array((W, H)), depth=255),
    )
    faces = np.array(((0, 1, 2), (1, 3, 2), (0, 2, 4), (0, 4, 3), (2, 5, 1)), np.int32)
    position = np.array(((0.0, 0.0, 0.0), (2.0, 0.0, 0.0), (0.0, 1.0, 0.0), (1.0, 1.0, 0.0), (-1, -1, 1.0), (-2, 0.0, 0.0)), F32)
    colour = np.array(((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 1.0), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (1.0, 1.0, 0.0)), F32)
    light_dir = np.array((0.0, 0.0, -1.0), F32)
    spec = JobSpec(shader=_lib.SHADER_GOURAUD, width=W, height=H, viewport=cam.viewport,
                   world_to_clip=cam.world_to_clip, world_to_eye_norm=cam.world_to_eye_norm,
                   position=position, faces=faces)
    spec.colour = colour
    spec.normal = np.tile(light_dir, (6, 1))
    spec.light_direction = light_dir
    spec.light_colour = np.ones(3, F32)
    return spec


def smoke_batched_triangles_asserts(zbuffer, canvas):
    """The assertions of tests/smoke_test.py:104-132 (x-major buffers in)."""
    from jaxrenderer_gb300.utils import transpose_for_display

    W, H = 1920, 1080
    z = transpose_for_display(np.asarray(zbuffer))
    c = transpose_for_display(np.asarray(canvas))
    assert z.shape == (H, W) and c.shape == (H, W, 3)
    assert np.unique(z[293:528, 964:1423].astype(np.uint8)).shape == (1,)
    assert np.all(z[590:1049, 964:1423] == 1.0)
    assert z[551, 914] < z[1026, 92]
    empty = (c == np.zeros(3, F32)).all(axis=2).sum()
    assert empty > (W * H // 2)
    assert empty < (W * H)


def specs_from_batch(flat, sb, s):
    """JobSpecs (depth pass, main pass) of scene s of a SceneBatch, for the oracle."""
    from jaxrenderer_gb300.batch import scene_job_specs

    return scene_job_specs(flat, sb, s)
