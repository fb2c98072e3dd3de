"""Gradients of the differentiable workload at its full per-scene size,
against masked FP64 central differences of the oracle (tests/fdgrad.py).

Scene (one of the 256 of the differentiable benchmark batch): a level-4
icosphere (5,120 triangles) with N(0, 0.05) displacement along the normal,
128 x 128 pixels, a 64 x 64 x 3 texture U[0, 1], a random unit light
direction, the camera at radius 4; loss = mean squared error against the
image of the undisplaced sphere.  The phong case is that workload's own
shader (PhongTextureShader, shaders/phong.py); the same scene also runs
through gouraud (shaders/gouraud.py:94-124), gouraud_texture
(shaders/gouraud_texture.py:107-144) and phong_reflection
(shaders/phong_reflection.py:158-235).  Each tensor the backward writes for
the shader is sampled at 64 random coordinates among the vertices of
visible faces and the texels that pixels sample, plus every component of
the light and camera inputs, and must agree with the FD to rtol 1e-3 (with
the FD-truncation and FP32 floors of tests/fdgrad.py).  The reference's own
gradient check is tests/smoke_test_grad.py:92-128.
"""
import os

import numpy as np
import pytest
import torch

from jaxrenderer_gb300 import _lib, batch as jb, synthetic
from jaxrenderer_gb300.autograd import DifferentiableBatch, camera_matrices
from jaxrenderer_gb300.geometry import Camera
from jaxrenderer_gb300.jobs import JobSpec
from oracle import oracle
from tests import fdgrad

pytestmark = pytest.mark.gpu
F32 = np.float32
W = H = 128
N_COORDS = 64
THREADS = max(1, len(os.sched_getaffinity(0)))

SHADERS = {
    "phong": _lib.SHADER_PHONG,
    "gouraud": _lib.SHADER_GOURAUD,
    "gouraud_texture": _lib.SHADER_GOURAUD_TEXTURE,
    "phong_reflection": _lib.SHADER_PHONG_REFLECTION,
}
# inputs of each shader that get gradients (RastGradPools / RAST_GRAD_*), besides the camera position
TENSORS = {
    "phong": ("position", "normal", "texture", "light_direction"),
    "gouraud": ("position", "normal", "colour", "light_direction", "light_colour"),
    "gouraud_texture": ("position", "normal", "texture", "light_direction", "light_colour"),
    "phong_reflection": ("position", "normal", "texture", "specular_map", "light_dir_eye", "ambient", "diffuse",
                         "specular", "light_colour"),
}
JOB_PARAMS = ("light_direction", "light_colour", "light_dir_eye", "ambient", "diffuse", "specular")


def camera64(eye, params):
    e = np.asarray(eye, np.float64)
    view = Camera.view_matrix(e, np.zeros(3), np.array((0.0, 0.0, 1.0)))
    vinv = Camera.view_matrix_inv(e, np.zeros(3), np.array((0.0, 0.0, 1.0)))
    aspect = np.tan(np.radians(params.hfov) / 2) / np.tan(np.radians(params.vfov) / 2)
    proj = Camera.perspective_projection_matrix(params.vfov, aspect, params.near, params.far, dtype=np.float64)
    vp = Camera.viewport_matrix(np.zeros(2, np.int32), np.array((W, H)), 1.0, dtype=np.float64)
    return Camera.create(view, proj, vp, vinv)


@pytest.fixture(scope="module")
def sphere():
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 4))
    sc = synthetic.phong_scene(rng, level=4, texture_size=64, sigma=0.05)
    extra = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 40))
    inputs = {
        "eye": sc.eye.astype(np.float64),
        "position": sc.position,
        "normal": sc.normal,
        "texture": sc.texture,
        "light_direction": sc.light_direction,
        "light_colour": np.array((0.9, 1.0, 0.8), F32),
        "colour": extra.uniform(0.05, 1.0, (len(sc.position), 3)).astype(F32),
        "specular_map": extra.uniform(1.0, 4.0, sc.texture.shape[:2]).astype(F32),
        "light_dir_eye": sc.light_direction,
        "ambient": np.array((0.3, 0.25, 0.2), F32),
        "diffuse": np.array((0.5, 0.6, 0.55), F32),
        "specular": np.array((0.4, 0.3, 0.5), F32),
    }
    return sc, inputs


def make_spec(kind, sc, x, dtype):
    params = synthetic.phong_camera_params(np.asarray(x["eye"], np.float64), W, H)
    cam = camera64(x["eye"], params)
    cast = lambda a: np.asarray(a, dtype)  # noqa: E731
    spec = JobSpec(shader=SHADERS[kind], width=W, height=H, viewport=cast(cam.viewport),
                   world_to_clip=cast(cam.world_to_clip), world_to_eye_norm=cast(cam.world_to_eye_norm),
                   position=cast(x["position"]), faces=sc.faces)
    spec.normal = cast(x["normal"])
    spec.light_direction = cast(x["light_direction"])
    spec.light_colour = cast(x["light_colour"])
    if kind == "gouraud":
        spec.colour = cast(x["colour"])
    if kind in ("phong", "gouraud_texture"):
        spec.uv = sc.uv  # texel units: these shaders floor uv directly
        spec.texture = cast(x["texture"])
    if kind == "phong_reflection":
        tw, th = x["texture"].shape[:2]
        spec.uv = (sc.uv / F32(tw)).astype(F32)  # [0, 1]: uv_repeat scales by the map's shape
        spec.texture = cast(x["texture"])
        spec.texture_shape = np.array([[tw, th]], np.int32)
        spec.texture_index = np.zeros(len(sc.position), np.int32)
        spec.texture_offset = tw
        spec.specular_map = cast(x["specular_map"])
        for k in ("light_dir_eye", "ambient", "diffuse", "specular"):
            setattr(spec, k, cast(x[k]))
    return spec


def oracle64(kind, sc, x, window=None):
    spec = make_spec(kind, sc, x, np.float64)
    return oracle.render(spec, np.ones((W, H)), np.ones((W, H, 3)), n_threads=THREADS, dtype=np.float64,
                         window=window, want_branch=True)


def analytic(kind, sc, x, M, target, device):
    """Gradients of sum(M * (canvas - target)^2) / N from the CUDA backward
    (tiled forward, rast_backward), through the torch camera twin for the
    camera position."""
    spec = make_spec(kind, sc, x, F32)
    sb = jb.scene_batch_from_specs([spec], device)
    db = DifferentiableBatch(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0))
    leaves = {}
    for name in TENSORS[kind]:
        a = np.asarray(x[name], F32)
        leaves[name] = torch.tensor(a[None] if name in JOB_PARAMS else a, requires_grad=True)
    eye = torch.tensor(np.asarray(x["eye"], np.float64)[None], requires_grad=True)
    params = synthetic.phong_camera_params(np.asarray(x["eye"], np.float64), W, H)
    w2c, w2e, _ = camera_matrices(eye, params)
    canvas, _ = db.render(world_to_clip=w2c.to(device, torch.float32), world_to_eye_norm=w2e.to(device, torch.float32),
                          **{k: v.to(device) for k, v in leaves.items()})
    m = torch.tensor(M, dtype=torch.float32, device=device)[None, ..., None]
    t = torch.tensor(target, dtype=torch.float32, device=device)[None]
    loss = (m * (canvas - t) ** 2).sum() / float(W * H * 3)
    loss.backward()
    out = {k: v.grad.numpy().reshape(np.asarray(x[k]).shape) for k, v in leaves.items()}
    out["eye"] = eye.grad.numpy()[0]
    return out, canvas[0].detach().cpu().numpy()


def coordinates(kind, sc, x, base, seed):
    """64 random coordinates per pool tensor among the vertices of faces
    that win lit pixels and the texels that lit pixels sample (the low bits
    of the oracle's branch signature are the shader's branch bits: bit 0 the
    lit / kept branch, bit 1 phong_reflection's specular branch), and every
    component of the light and camera inputs."""
    rng = np.random.Generator(np.random.PCG64(seed))
    prim, texel, bits = base["prim_id"], base["texel"], base["branch"] & 15
    lit = (prim >= 0) & ((bits & 1) != 0)
    vis_verts = np.unique(sc.faces[np.unique(prim[lit])].reshape(-1))
    coords = [fdgrad.Coord("eye", k) for k in range(3)]
    for name in TENSORS[kind]:
        if name in ("position", "normal", "colour"):
            verts = rng.choice(vis_verts, N_COORDS, replace=False)
            win = fdgrad.vertex_windows(sc.faces, prim, verts)
            coords += [fdgrad.Coord(name, 3 * int(v) + int(rng.integers(3)), win[int(v)]) for v in verts]
        elif name in ("texture", "specular_map"):
            active = lit & ((bits & 2) != 0) if name == "specular_map" else lit
            used = np.unique(texel[active])
            rows = rng.choice(used, N_COORDS, replace=False)
            win = fdgrad.texel_windows(texel, rows)
            per = 3 if name == "texture" else 1
            coords += [fdgrad.Coord(name, per * int(r) + int(rng.integers(per)), win[int(r)]) for r in rows]
        else:
            coords += [fdgrad.Coord(name, k) for k in range(3)]
    return coords


@pytest.mark.parametrize("kind", list(SHADERS))
def test_gradients_at_full_size_vs_fd64(cuda_device, sphere, kind):
    sc, x32 = sphere
    x = {k: np.asarray(v, np.float64) for k, v in x32.items()}
    undisplaced = dict(x, position=np.asarray(sc.base_position, np.float64))
    target = oracle64(kind, sc, undisplaced)["canvas"].astype(F32).astype(np.float64)
    base = oracle64(kind, sc, x)
    covered = base["prim_id"] >= 0
    assert covered.sum() > 2000
    coords = coordinates(kind, sc, x, base, seed=100 + SHADERS[kind])
    M, results = fdgrad.masked_fd(lambda p, win: oracle64(kind, sc, p, win), x, coords, base, target)
    assert M.sum() >= 0.75 * covered.sum(), (M.sum(), covered.sum())
    grads, canvas = analytic(kind, sc, x, M, target, cuda_device)
    # forward agreement on M (FP32 kernel vs FP64 oracle): the gradients are of the same function
    assert np.abs(canvas - base["canvas"])[M].max() < 1e-4
    stats = fdgrad.compare(results, grads)
    for name, s in stats.items():
        assert s["nonzero"] >= 0.75 * s["n"], (name, s)  # the check is not vacuous
    # per tensor: coordinates, within rtol 1e-3 with no floor, max relative error vs the eps = 1e-3 FD and
    # vs its Richardson extrapolation, max error / bound
    print(kind, {k: (v["n"], v["within_rtol"], f'{v["max_rel"]:.1e}', f'{v["max_rel_richardson"]:.1e}',
                     round(v["max_err_over_bound"], 3)) for k, v in stats.items()})
