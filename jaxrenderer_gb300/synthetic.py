"""Seeded synthetic scenes for the benchmark workloads and the parity tests.

The reference benchmarks on Brax Ant scenes it renders in notebooks; the
workloads here are seeded stand-ins with the stated shapes: a ground plane
plus 8-32 objects drawn from {box 12 tris, icosphere level 2 (320 tris),
capsule 16x8 segments (~512 tris)} per 84x84 scene, and so on.  Generators
use numpy's PCG64 with seed 20230701 + workload index.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from .geometry import Camera, transform_matrix_from_rotation
from .model import Model, ModelObject
from .shapes.cube import create_cube

F32 = np.float32
BASE_SEED = 20230701


def icosphere(level: int) -> Tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: 20 * 4**level faces, shared vertices, CCW outward."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
         (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, dtype=np.float64) / np.linalg.norm(p) for p in v]
    faces = list(f)
    for _ in range(level):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.asarray(verts, dtype=F32), np.asarray(faces, dtype=np.int32)


def sphere_uv(verts: np.ndarray) -> np.ndarray:
    u = 0.5 + np.arctan2(verts[:, 1], verts[:, 0]) / (2 * np.pi)
    w = 0.5 + np.arcsin(np.clip(verts[:, 2], -1, 1)) / np.pi
    return np.stack([u, w], axis=1).astype(F32)


def capsule_mesh(segments: int = 16, rings: int = 8, half_height: float = 0.5) -> Tuple[np.ndarray, np.ndarray]:
    """Capsule with `segments` around and `rings` latitude bands per hemisphere
    plus a cylinder band; pole bands are fans: 16x8 -> 512 triangles."""
    verts = []
    lat = []
    for r in range(rings + 1):  # north hemisphere, pole to equator
        lat.append((np.pi / 2 * r / rings, +half_height))
    for r in range(rings + 1):  # south hemisphere, equator to pole
        lat.append((np.pi / 2 + np.pi / 2 * r / rings, -half_height))
    for theta, dz in lat:
        for s in range(segments):
            phi = 2 * np.pi * s / segments
            verts.append((np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta) + dz))
    faces = []
    nrow = len(lat)
    for r in range(nrow - 1):
        for s in range(segments):
            a = r * segments + s
            b = r * segments + (s + 1) % segments
            c = (r + 1) * segments + s
            d = (r + 1) * segments + (s + 1) % segments
            if r == 0:  # north pole fan
                faces.append((a, c, d))
            elif r == nrow - 2:  # south pole fan
                faces.append((a, c, b))
            else:
                faces.append((a, c, d))
                faces.append((a, d, b))
    return np.asarray(verts, dtype=F32), np.asarray(faces, dtype=np.int32)


def _normals_of(verts: np.ndarray, centre_z: Optional[np.ndarray] = None) -> np.ndarray:
    n = verts.astype(np.float64).copy()
    if centre_z is not None:
        n[:, 2] -= centre_z
    return (n / np.linalg.norm(n, axis=1, keepdims=True)).astype(F32)


_PRIMS = {}


def primitive_model(kind: str, colour: np.ndarray, specular: float = 2.0) -> Model:
    """One of the workload primitives with a 4x4 texture of `colour`."""
    tex = np.broadcast_to(np.asarray(colour, F32), (4, 4, 3)).copy()
    spec = np.full((4, 4), specular, F32)
    if kind == "box":
        return create_cube(np.ones(3, F32) * 0.5, np.ones(2, F32), tex, spec)
    if kind not in _PRIMS:
        if kind == "icosphere2":
            v, f = icosphere(2)
            v = v * F32(0.5)
            _PRIMS[kind] = (v, _normals_of(v), sphere_uv(v), f)
        elif kind == "capsule":
            v, f = capsule_mesh(16, 8, 0.5)
            cz = np.where(v[:, 2] > 0, 0.5, -0.5).astype(np.float64)
            n = _normals_of(v, cz)
            v = v * F32(0.4)
            _PRIMS[kind] = (v.astype(F32), n, sphere_uv(n), f)
        else:
            raise ValueError(kind)
    v, n, uv, f = _PRIMS[kind]
    return Model(verts=v, norms=n, uvs=uv, faces=f, faces_norm=f, faces_uv=f, diffuse_map=tex, specular_map=spec)


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    q = rng.normal(size=4)
    q = q / np.linalg.norm(q)
    return transform_matrix_from_rotation(q.astype(F32))


@dataclass
class BraxLikeScene:
    objects: List[ModelObject]
    camera_position: np.ndarray
    n_faces: int


def brax_like_scene(rng: np.random.Generator) -> BraxLikeScene:
    """Ground plane (2 triangles, 10x10) plus 8..32 random objects, camera on
    a radius-6 sphere at elevation U[20, 60] deg, azimuth U[0, 360) deg."""
    objects = []
    ground_tex = np.broadcast_to(rng.uniform(0, 1, 3).astype(F32), (4, 4, 3)).copy()
    gv = np.array([(-5, -5, 0), (5, -5, 0), (5, 5, 0), (-5, 5, 0)], F32)
    gf = np.array([(0, 1, 2), (0, 2, 3)], np.int32)
    gn = np.tile(np.array([(0, 0, 1)], F32), (4, 1))
    guv = np.array([(0, 0), (4, 0), (4, 4), (0, 4)], F32)
    ground = Model(gv, gn, guv, gf, gf, gf, ground_tex, np.full((4, 4), 2.0, F32))
    objects.append(ModelObject(model=ground))
    n_obj = int(rng.integers(8, 33))
    kinds = ("box", "icosphere2", "capsule")
    nf = 2
    for _ in range(n_obj):
        kind = kinds[int(rng.integers(0, 3))]
        model = primitive_model(kind, rng.uniform(0, 1, 3))
        t = np.identity(4, dtype=F32)
        t[:3, :3] = random_rotation(rng)
        t[:3, 3] = (rng.uniform(-3, 3), rng.uniform(-3, 3), rng.uniform(0, 2))
        s = F32(rng.uniform(0.2, 1.0))
        objects.append(ModelObject(model=model, local_scaling=np.full(3, s, F32), transform=t))
        nf += len(model.faces)
    elev = np.deg2rad(rng.uniform(20, 60))
    azim = np.deg2rad(rng.uniform(0, 360))
    pos = 6.0 * np.array([np.cos(elev) * np.cos(azim), np.cos(elev) * np.sin(azim), np.sin(elev)])
    return BraxLikeScene(objects=objects, camera_position=pos.astype(F32), n_faces=nf)


def random_triangle_soup(rng: np.random.Generator, n_faces: int, spread: float = 1.5,
                         size: float = 0.6, shared: bool = False) -> Tuple[np.ndarray, np.ndarray]:
    """Random triangles around the origin, some crossing z = camera planes,
    with duplicates (exact depth ties) and degenerate ones mixed in."""
    centres = rng.uniform(-spread, spread, size=(n_faces, 1, 3))
    offs = rng.normal(scale=size, size=(n_faces, 3, 3))
    tri = (centres + offs).astype(F32)
    if n_faces >= 8:
        k = max(1, n_faces // 16)
        tri[-k:] = tri[:k]  # exact duplicates: ties resolved by lowest id
        tri[k, 2] = tri[k, 1]  # degenerate (zero area)
    verts = tri.reshape(-1, 3)
    faces = np.arange(verts.shape[0], dtype=np.int32).reshape(-1, 3)
    return verts, faces


__all__ = [
    "icosphere",
    "capsule_mesh",
    "primitive_model",
    "brax_like_scene",
    "random_triangle_soup",
    "BASE_SEED",
]


# --------------------------------------------------- batched Brax-like workload

_KINDS = ("box", "icosphere2", "capsule")


def _base_mesh(kind: str):
    m = primitive_model(kind, np.zeros(3, F32))
    return np.asarray(m.verts, F32), np.asarray(m.norms, F32), np.asarray(m.uvs, F32), np.asarray(m.faces, np.int32)


@dataclass
class FlatScenes:
    """Many merged scenes, flattened per face corner, in flat arrays.

    Scene s owns corner rows [corner_begin[s], corner_begin[s] + 3 * n_faces[s])
    of position/normal/uv/texture_index, faces 3 * arange within them, and
    texture rows [tex_begin[s], tex_begin[s] + T * n_objects[s]) of the
    T x T diffuse (RGB) maps, T = tex_size, and the matching rows of the
    specular maps (spec_size, default T).  Maps smaller than T are padded
    with zeros at the end of each axis (merge_maps) and keep their own size
    in texture_shape.
    """

    position: np.ndarray
    normal: np.ndarray
    uv: np.ndarray
    texture_index: np.ndarray
    texture: np.ndarray
    specular_map: np.ndarray
    corner_begin: np.ndarray
    n_faces: np.ndarray
    tex_begin: np.ndarray
    n_objects: np.ndarray
    camera_position: np.ndarray
    tex_size: int = 4  # every object's diffuse map is padded to tex_size x tex_size
    camera_target: Optional[np.ndarray] = None  # (N, 3); origin when None
    texture_shape: Optional[np.ndarray] = None  # (objects, 2): maps' own sizes; tex_size when None
    spec_size: Optional[int] = None  # specular maps padded to spec_size^2; tex_size when None

    @property
    def n_scenes(self) -> int:
        return int(self.n_faces.shape[0])


def brax_like_batch(n_scenes: int, seed: int = BASE_SEED + 1) -> FlatScenes:
    """`n_scenes` Brax-like scenes (see brax_like_scene), already merged and
    flattened per face corner.  Object vertices are scaled, rotated and
    translated; normals go through the rotation (the inverse-transpose of a
    rotation times a uniform scale, normalised per vertex)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    bases = {k: _base_mesh(k) for k in _KINDS}
    gv = np.array([(-5, -5, 0), (5, -5, 0), (5, 5, 0), (-5, 5, 0)], F32)
    gf = np.array([(0, 1, 2), (0, 2, 3)], np.int32)
    guv = np.array([(0, 0), (4, 0), (4, 4), (0, 4)], F32)
    n_obj = rng.integers(8, 33, size=n_scenes)
    kinds = [rng.integers(0, 3, size=int(k)) for k in n_obj]
    quats = [rng.normal(size=(int(k), 4)) for k in n_obj]
    trans = [np.stack([rng.uniform(-3, 3, int(k)), rng.uniform(-3, 3, int(k)), rng.uniform(0, 2, int(k))], 1) for k in n_obj]
    scales = [rng.uniform(0.2, 1.0, int(k)) for k in n_obj]
    colours = [rng.uniform(0, 1, (int(k) + 1, 3)) for k in n_obj]
    elev = np.deg2rad(rng.uniform(20, 60, n_scenes))
    azim = np.deg2rad(rng.uniform(0, 360, n_scenes))
    cam = 6.0 * np.stack([np.cos(elev) * np.cos(azim), np.cos(elev) * np.sin(azim), np.sin(elev)], 1)
    face_counts = {k: bases[k][3].shape[0] for k in _KINDS}
    n_faces = np.array([2 + sum(face_counts[_KINDS[int(t)]] for t in ks) for ks in kinds], np.int64)
    corner_begin = np.concatenate([[0], np.cumsum(3 * n_faces)[:-1]]).astype(np.int64)
    total = int(3 * n_faces.sum())
    position = np.empty((total, 3), F32)
    normal = np.empty((total, 3), F32)
    uv = np.empty((total, 2), F32)
    tex_idx = np.empty(total, np.int32)
    objs = n_obj + 1
    tex_begin = np.concatenate([[0], np.cumsum(4 * objs)[:-1]]).astype(np.int64)
    texture = np.empty((int(4 * objs.sum()), 4, 3), F32)
    specular = np.full((int(4 * objs.sum()), 4), 2.0, F32)
    for s in range(n_scenes):
        row = corner_begin[s]
        corners = gv[gf.reshape(-1)]
        position[row : row + 6] = corners
        normal[row : row + 6] = (0, 0, 1)
        uv[row : row + 6] = guv[gf.reshape(-1)]
        tex_idx[row : row + 6] = 0
        row += 6
        q = quats[s] / np.linalg.norm(quats[s], axis=1, keepdims=True)
        for o, t in enumerate(kinds[s]):
            v, n, u, f = bases[_KINDS[int(t)]]
            R = transform_matrix_from_rotation(q[o].astype(F32)).astype(F32)
            sc = F32(scales[s][o])
            idx = f.reshape(-1)
            p = (v[idx] * sc) @ R.T + trans[s][o].astype(F32)
            nn = n[idx] @ R.T
            nn = nn / np.linalg.norm(nn, axis=1, keepdims=True)
            k = idx.size
            position[row : row + k] = p
            normal[row : row + k] = nn
            uv[row : row + k] = u[idx]
            tex_idx[row : row + k] = o + 1
            row += k
        tb = tex_begin[s]
        texture[tb : tb + 4 * objs[s]] = np.repeat(colours[s], 4, axis=0)[:, None, :].astype(F32)
    return FlatScenes(position, normal, uv, tex_idx, texture, specular, corner_begin, n_faces.astype(np.int32),
                      tex_begin, objs.astype(np.int32), cam.astype(F32))


# ------------------------------------------------ differentiable phong batch

@dataclass
class PhongScene:
    """One scene of the differentiable phong workload (PhongTextureShader)."""

    base_position: np.ndarray  # (V, 3) unperturbed icosphere
    position: np.ndarray  # (V, 3) displaced along the normal
    normal: np.ndarray
    uv: np.ndarray  # texel units
    faces: np.ndarray
    texture: np.ndarray  # (tw, th, 3)
    light_direction: np.ndarray  # eye space
    eye: np.ndarray  # camera position


def phong_scene(rng: np.random.Generator, level: int = 4, texture_size: int = 64, sigma: float = 0.05,
                radius: float = 4.0) -> PhongScene:
    """Icosphere of `level` with per-vertex Gaussian displacement sigma along
    the normal, a texture_size^2 RGB texture U[0, 1] sampled in texel units,
    a random unit light direction (eye space, towards the viewer's side) and
    a camera on a sphere of `radius` looking at the origin."""
    v, f = icosphere(level)
    n = v.copy()
    disp = rng.normal(0.0, sigma, size=(len(v), 1)).astype(F32)
    pos = (v * (F32(1) + disp)).astype(F32)
    uv = (sphere_uv(v) * F32(texture_size)).astype(F32)
    tex = rng.uniform(0, 1, (texture_size, texture_size, 3)).astype(F32)
    l = rng.normal(size=3)
    l[2] = abs(l[2]) + 0.5
    l = (l / np.linalg.norm(l)).astype(F32)
    e = rng.normal(size=3)
    e = (radius * e / np.linalg.norm(e)).astype(F32)
    return PhongScene(v, pos, n, uv, f, tex, l, e)


def phong_camera_params(eye, width: int = 128, height: int = 128):
    """Camera of the differentiable phong workload: at `eye`, looking at the
    origin, +Z up, 40 degree field of view, near 0.1, far 100."""
    from .renderer import CameraParameters

    return CameraParameters(viewWidth=width, viewHeight=height, near=0.1, far=100.0, hfov=40.0, vfov=40.0,
                            position=np.asarray(eye, F32), target=np.zeros(3, F32))


def phong_job_spec(sc: PhongScene, width: int = 128, height: int = 128, position: Optional[np.ndarray] = None):
    """JobSpec of PhongTextureShader (phong.py) rendering `sc` (its displaced
    positions unless `position` is given) through phong_camera_params."""
    from . import _lib
    from .jobs import JobSpec
    from .renderer import Renderer

    cam = Renderer.create_camera_from_parameters(phong_camera_params(sc.eye, width, height))
    spec = JobSpec(shader=_lib.SHADER_PHONG, width=width, height=height, viewport=cam.viewport,
                   world_to_clip=cam.world_to_clip, world_to_eye_norm=cam.world_to_eye_norm,
                   position=np.asarray(sc.position if position is None else position, F32), faces=sc.faces)
    spec.normal = sc.normal
    spec.uv = sc.uv
    spec.texture = sc.texture
    spec.light_direction = sc.light_direction
    spec.light_colour = np.ones(3, F32)
    return spec


# ------------------------------------------- large overlapping single scene

def overdraw_scene(rng: np.random.Generator, width: int = 960, height: int = 540,
                   n_l4: int = 64, n_l5: int = 3, texture_size: int = 512):
    """Single gouraud_texture scene of 64 level-4 + 3 level-5 icospheres
    (389,120 triangles) at random overlapping placements in front of the
    camera, a 512x512x3 U[0, 1] texture sampled in texel units, and a few
    exact duplicate spheres (equal depths: ties resolved by lowest index).
    Returns (JobSpec fields as a dict, estimated mean overdraw)."""
    from .geometry import Camera

    meshes = []
    v4, f4 = icosphere(4)
    v5, f5 = icosphere(5)
    positions, normals, uvs, faces = [], [], [], []
    offset = 0
    centres, radii = [], []
    kinds = [4] * n_l4 + [5] * n_l5
    for k, lvl in enumerate(kinds):
        v, f = (v4, f4) if lvl == 4 else (v5, f5)
        if k >= 4 and k % 16 == 0:
            c, r = centres[k - 4], radii[k - 4]  # exact duplicate of an earlier sphere
        else:
            c = rng.uniform((-2.2, -1.2, -1.5), (2.2, 1.2, 1.5))
            r = rng.uniform(2.2, 3.6)
        centres.append(c)
        radii.append(r)
        p = (v.astype(np.float64) * r + c).astype(F32)
        positions.append(p)
        normals.append(v.copy())
        uvs.append((sphere_uv(v) * texture_size * rng.uniform(0.5, 2.0)).astype(F32))
        faces.append(f + offset)
        offset += len(v)
    eye = np.array((0.0, 0.0, 9.0), F32)
    view = Camera.view_matrix(eye, np.zeros(3, F32), np.array((0, 1, 0), F32))
    proj = Camera.perspective_projection_matrix(45.0, width / height, 0.1, 100.0)
    vp = Camera.viewport_matrix(np.zeros(2, np.int32), np.array((width, height)), 1.0)
    cam = Camera.create(view, proj, vp)
    # projected disc area estimate: f_px * r / depth
    fpx = (height / 2) / np.tan(np.radians(22.5))
    area = sum(np.pi * (fpx * r / (9.0 - c[2])) ** 2 for c, r in zip(centres, radii))
    light = rng.normal(size=3)
    light = (light / np.linalg.norm(light)).astype(F32)
    spec = dict(
        width=width, height=height, viewport=cam.viewport, world_to_clip=cam.world_to_clip,
        world_to_eye_norm=cam.world_to_eye_norm, position=np.concatenate(positions),
        normal=np.concatenate(normals), uv=np.concatenate(uvs), faces=np.concatenate(faces).astype(np.int32),
        texture=rng.uniform(0, 1, (texture_size, texture_size, 3)).astype(F32),
        light_direction=-light if light[2] < 0 else light, light_colour=np.ones(3, F32),
    )
    return spec, float(area / (width * height))


def _quat_matrices(q: np.ndarray) -> np.ndarray:
    """(K, 3, 3) rotation matrices of (K, 4) unit (w, x, y, z) quaternions,
    the same convention as geometry.transform_matrix_from_rotation."""
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
    ], -2)


def cube_scene_batch(n_scenes: int, seed: int = BASE_SEED + 5, f_min: int = 100, f_max: int = 100_000,
                     chunk: int = 65536) -> FlatScenes:
    """Scenes built from the config-1 primitive (create_cube, 12 triangles,
    24 vertices with normals and UVs): triangle counts log-uniform in
    [f_min, f_max] (rounded to whole cubes), cubes at uniform positions in a
    box of half-extent 1.5 * cubes^(1/3), random unit-quaternion rotations,
    scales U[0.3, 0.8], one RGB diffuse U[0, 1] per cube on a 4x4 map,
    specular 2.0; the camera at 3.2 half-extents on a random direction above
    the box's mid-plane, looking at the origin."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cube = create_cube(np.ones(3, F32), np.ones(2, F32), np.zeros((4, 4, 3), F32), np.full((4, 4), 2.0, F32))
    idx = np.asarray(cube.faces, np.int32).reshape(-1)
    cv = np.asarray(cube.verts, F32)[idx]
    cn = np.asarray(cube.norms, F32)[idx]
    cu = np.asarray(cube.uvs, F32)[idx]
    n_cubes = np.maximum(1, np.round(np.exp(rng.uniform(np.log(f_min), np.log(f_max), n_scenes)) / 12)).astype(np.int64)
    K = int(n_cubes.sum())
    scene_of = np.repeat(np.arange(n_scenes), n_cubes)
    half = 1.5 * n_cubes.astype(np.float64) ** (1.0 / 3.0)
    centres = rng.uniform(-1.0, 1.0, (K, 3)) * half[scene_of, None]
    q = rng.normal(size=(K, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    scale = rng.uniform(0.3, 0.8, K)
    colour = rng.uniform(0, 1, (K, 3))
    d = rng.normal(size=(n_scenes, 3))
    d[:, 2] = np.abs(d[:, 2]) + 0.3
    cams = (3.2 * half[:, None] * d / np.linalg.norm(d, axis=1, keepdims=True)).astype(F32)
    position = np.empty((36 * K, 3), F32)
    normal = np.empty((36 * K, 3), F32)
    for a in range(0, K, chunk):
        b = min(K, a + chunk)
        R = _quat_matrices(q[a:b])
        position[36 * a : 36 * b] = (np.einsum("kij,vj->kvi", R * scale[a:b, None, None], cv)
                                     + centres[a:b, None, :]).reshape(-1, 3)
        normal[36 * a : 36 * b] = np.einsum("kij,vj->kvi", R, cn).reshape(-1, 3)
    uv = np.tile(cu, (K, 1))
    cube_begin = np.concatenate([[0], np.cumsum(n_cubes)[:-1]])
    tex_idx = (np.arange(K, dtype=np.int64) - cube_begin[scene_of]).astype(np.int32).repeat(36)
    texture = np.repeat(colour, 4, axis=0)[:, None, :].repeat(4, axis=1).astype(F32)
    specular = np.full((4 * K, 4), 2.0, F32)
    n_faces = (12 * n_cubes).astype(np.int32)
    corner_begin = 36 * cube_begin
    return FlatScenes(position, normal, uv, tex_idx, texture, specular, corner_begin.astype(np.int64), n_faces,
                      (4 * cube_begin).astype(np.int64), n_cubes.astype(np.int32), cams, 4,
                      np.zeros((n_scenes, 3), F32))


def flat_subset(flat: FlatScenes, scenes: Sequence[int]) -> FlatScenes:
    """The scenes `scenes` of a FlatScenes batch as a FlatScenes of their own
    (corner and texture rows gathered, offsets rebased)."""
    sel = np.asarray(scenes, np.int64)
    T = flat.tex_size
    Ts = flat.spec_size or T
    nf = flat.n_faces[sel].astype(np.int64)
    no = flat.n_objects[sel].astype(np.int64)
    ob = np.concatenate([[0], np.cumsum(flat.n_objects.astype(np.int64))])[sel]
    cat = lambda parts: np.concatenate(parts) if len(parts) else np.zeros(0, np.int64)  # noqa: E731
    rows = cat([np.arange(c, c + 3 * f) for c, f in zip(flat.corner_begin[sel], nf)])
    trows = cat([np.arange(b * T, (b + o) * T) for b, o in zip(ob, no)])
    srows = cat([np.arange(b * Ts, (b + o) * Ts) for b, o in zip(ob, no)])
    objs = cat([np.arange(b, b + o) for b, o in zip(ob, no)])
    corner_begin = np.concatenate([[0], np.cumsum(3 * nf)[:-1]]).astype(np.int64)
    tex_begin = np.concatenate([[0], np.cumsum(T * no)[:-1]]).astype(np.int64)
    target = None if flat.camera_target is None else flat.camera_target[sel]
    shapes = None if flat.texture_shape is None else np.asarray(flat.texture_shape)[objs]
    return FlatScenes(flat.position[rows], flat.normal[rows], flat.uv[rows], flat.texture_index[rows],
                      flat.texture[trows], flat.specular_map[srows], corner_begin, flat.n_faces[sel].copy(),
                      tex_begin, flat.n_objects[sel].copy(), flat.camera_position[sel].copy(), T, target, shapes,
                      flat.spec_size)


def brax_like_instances(n_scenes: int, seed: int = BASE_SEED + 1):
    """`n_scenes` Brax-like scenes as instances of four meshes (ground plane,
    box, level-2 icosphere, 16x8 capsule): the ground (identity transform)
    plus 8..32 objects with ModelObject transforms [R | t] (random unit
    quaternion, t in [-3, 3]^2 x [0, 2]), uniform local scaling U[0.2, 1],
    one RGB colour U[0, 1] per object on a 4x4 map, specular 2.0; camera on a
    radius-6 sphere at elevation U[20, 60] deg, azimuth U[0, 360) deg."""
    from .instancing import InstancedScenes, MeshLibrary

    rng = np.random.Generator(np.random.PCG64(seed))
    gv = np.array([(-5, -5, 0), (5, -5, 0), (5, 5, 0), (-5, 5, 0)], F32)
    gf = np.array([(0, 1, 2), (0, 2, 3)], np.int32)
    gn = np.tile(np.array([(0, 0, 1)], F32), (4, 1))
    guv = np.array([(0, 0), (4, 0), (4, 4), (0, 4)], F32)
    blank = np.zeros((4, 4, 3), F32)
    ground = Model(gv, gn, guv, gf, gf, gf, blank, np.full((4, 4), 2.0, F32))
    library = MeshLibrary.from_models([ground] + [primitive_model(k, np.zeros(3, F32)) for k in _KINDS])
    n_obj = rng.integers(8, 33, size=n_scenes)
    counts = n_obj + 1
    I = int(counts.sum())
    scene_begin = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    is_ground = np.zeros(I, bool)
    is_ground[scene_begin[:-1]] = True
    mesh = np.zeros(I, np.int32)
    mesh[~is_ground] = 1 + rng.integers(0, 3, size=I - n_scenes)
    q = rng.normal(size=(I, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    transforms = np.tile(np.identity(4, F32), (I, 1, 1))
    transforms[~is_ground, :3, :3] = _quat_matrices(q[~is_ground]).astype(F32)
    k = I - n_scenes
    transforms[~is_ground, :3, 3] = np.stack([rng.uniform(-3, 3, k), rng.uniform(-3, 3, k), rng.uniform(0, 2, k)],
                                             1).astype(F32)
    scale = np.ones((I, 3), F32)
    scale[~is_ground] = rng.uniform(0.2, 1.0, (k, 1)).astype(F32)
    colour = rng.uniform(0, 1, (I, 3)).astype(F32)
    diffuse = np.broadcast_to(colour[:, None, None, :], (I, 4, 4, 3)).copy()
    specular = np.full((I, 4, 4), 2.0, F32)
    elev = np.deg2rad(rng.uniform(20, 60, n_scenes))
    azim = np.deg2rad(rng.uniform(0, 360, n_scenes))
    cam = 6.0 * np.stack([np.cos(elev) * np.cos(azim), np.cos(elev) * np.sin(azim), np.sin(elev)], 1)
    return InstancedScenes(library, mesh, scene_begin, transforms, scale, diffuse, specular, cam.astype(F32))


def ant_like_batched(n_frames: int, seed: int = BASE_SEED + 7):
    """A stand-in for the reference's pickled Brax Ant batches, in their
    format (see brax.load_batched_inputs): 18 objects per frame -- a box
    ground of 12 triangles with a 100x100 checker texture and 17 capsules of
    192 triangles with 1x1 maps (3,276 triangles) -- each array with a
    leading frame axis; objects move between frames, meshes do not; camera
    960x540, hfov 58, vfov 32.625, circling the moving target."""
    from .renderer import CameraParameters
    from .shapes.capsule import create_capsule

    rng = np.random.Generator(np.random.PCG64(seed))
    F = n_frames
    check = ((np.indices((100, 100)).sum(0) // 10) % 2).astype(F32)
    tex = np.stack([0.25 + 0.5 * check, 0.3 + 0.4 * check, 0.35 + 0.3 * check], -1).astype(F32)
    ground = create_cube(np.array((1000.0, 1000.0, 1e-4), F32), np.array((1000.0, 1000.0), F32) / 100.0, tex,
                         np.full((1, 1), 2.0, F32))
    caps = [create_capsule(F32(r), F32(h), 2, np.array([[[0.4, 0.33, 0.26]]], F32), np.full((1, 1), 2.0, F32))
            for r, h in zip(rng.uniform(0.06, 0.12, 17), rng.uniform(0.1, 0.25, 17))]
    models = [ground] + caps

    def batched(a):
        return np.broadcast_to(np.asarray(a), (F,) + np.asarray(a).shape).copy()

    centre = np.cumsum(rng.normal(0, 0.05, (F, 3)), axis=0).astype(F32)
    centre[:, 2] = 0.0
    objects = []
    for k, m in enumerate(models):
        model = Model(*(batched(x) for x in m))
        T = np.tile(np.identity(4, F32), (F, 1, 1))
        if k > 0:
            q = rng.normal(size=(F, 4))
            q /= np.linalg.norm(q, axis=1, keepdims=True)
            T[:, :3, :3] = _quat_matrices(q)
            T[:, :3, 3] = centre + rng.normal(0, 0.35, (F, 3)).astype(F32) * np.array((1, 1, 0.3), F32)
            T[:, 2, 3] = np.abs(T[:, 2, 3]) + 0.2
        objects.append(ModelObject(model=model, local_scaling=batched(np.ones(3, F32)), transform=T,
                                   double_sided=np.zeros(F, bool)))
    ang = np.linspace(0, np.pi / 2, F) + rng.uniform(0, 2 * np.pi)
    pos = centre + np.stack([3.7 * np.cos(ang), 3.7 * np.sin(ang), np.full(F, 1.9)], 1).astype(F32)
    camera = CameraParameters(viewWidth=np.full(F, 960, np.int32), viewHeight=np.full(F, 540, np.int32),
                              viewDepth=np.ones(F, F32), near=np.full(F, 0.01, F32), far=np.full(F, 1000.0, F32),
                              hfov=np.full(F, 58.0, F32), vfov=np.full(F, 32.625, F32), position=pos.astype(F32),
                              target=centre, up=batched(np.array((0, 0, 1), F32)))
    return objects, camera, centre.copy()
