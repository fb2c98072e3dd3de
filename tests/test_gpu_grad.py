"""GPU gradients (rast_backward through DifferentiableBatch) against central
finite differences of the FP64 oracle, eps 1e-3.  Pixels whose winning
primitive changes under +-eps are masked out of both sides (visibility is
piecewise constant, as under jax.grad of the reference)."""
import numpy as np
import pytest
import torch

import jaxrenderer_gb300 as jr
from jaxrenderer_gb300 import _lib, batch as jb, synthetic
from jaxrenderer_gb300.autograd import DifferentiableBatch, camera_matrices
from jaxrenderer_gb300.geometry import Camera
from jaxrenderer_gb300.jobs import JobSpec
from oracle import oracle

pytestmark = pytest.mark.gpu
F32 = np.float32
EPS = 1e-3
W = H = 48


def cam_params(eye):
    return jr.CameraParameters(viewWidth=W, viewHeight=H, near=0.1, far=100.0, hfov=40.0, vfov=40.0,
                               position=np.asarray(eye, F32), target=np.zeros(3, F32))


def camera64(eye, params):
    e = np.asarray(eye, np.float64)
    view = Camera.view_matrix(e, np.zeros(3), np.array((0.0, 0.0, 1.0)))
    vinv = Camera.view_matrix_inv(e, np.zeros(3), np.array((0.0, 0.0, 1.0)))
    aspect = np.tan(np.radians(params.hfov) / 2) / np.tan(np.radians(params.vfov) / 2)
    proj = Camera.perspective_projection_matrix(params.vfov, aspect, params.near, params.far, dtype=np.float64)
    vp = Camera.viewport_matrix(np.zeros(2, np.int32), np.array((W, H)), 1.0, dtype=np.float64)
    return Camera.create(view, proj, vp, vinv)


def phong_spec(sc, eye, light, position, texture, dtype=F32):
    params = cam_params(sc.eye)
    cam = camera64(eye, params)
    cast = lambda a: np.asarray(a, dtype)  # noqa: E731
    spec = JobSpec(shader=_lib.SHADER_PHONG, width=W, height=H, viewport=cast(cam.viewport),
                   world_to_clip=cast(cam.world_to_clip), world_to_eye_norm=cast(cam.world_to_eye_norm),
                   position=cast(position), faces=sc.faces)
    spec.normal = cast(sc.normal)
    spec.uv = sc.uv
    spec.texture = cast(texture)
    spec.light_direction = cast(light)
    spec.light_colour = np.ones(3, dtype)
    return spec


def oracle_loss(spec, target, mask):
    out = oracle.render(spec, np.ones((W, H), np.float64), np.ones((W, H, 3), np.float64), dtype=np.float64)
    d = out["canvas"] - target
    return float((mask[..., None] * d * d).sum()), out["prim_id"]


@pytest.fixture(scope="module")
def scene():
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 4))
    return synthetic.phong_scene(rng, level=2, texture_size=16, sigma=0.05)


def analytic(scene, mask, target, texture, cuda_device):
    sc = scene
    params = cam_params(sc.eye)
    spec = phong_spec(sc, sc.eye, sc.light_direction, sc.position, texture)
    sb = jb.scene_batch_from_specs([spec], cuda_device)
    db = DifferentiableBatch(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0))
    eye = torch.tensor(sc.eye, dtype=torch.float64, requires_grad=True)
    light = torch.tensor(sc.light_direction[None], dtype=torch.float32, requires_grad=True)
    pos = torch.tensor(sc.position, dtype=torch.float32, requires_grad=True)
    tex = torch.tensor(texture, dtype=torch.float32, requires_grad=True)
    w2c, w2e, _ = camera_matrices(eye[None], params)
    canvas, _ = db.render(position=pos.to(cuda_device), texture=tex.to(cuda_device),
                          world_to_clip=w2c.to(cuda_device, torch.float32),
                          world_to_eye_norm=w2e.to(cuda_device, torch.float32),
                          light_direction=light.to(cuda_device))
    m = torch.tensor(mask, dtype=torch.float32, device=cuda_device)[None, ..., None]
    t = torch.tensor(target, dtype=torch.float32, device=cuda_device)[None]
    loss = (m * (canvas - t) ** 2).sum()
    loss.backward()
    return eye.grad.numpy(), light.grad.numpy()[0], pos.grad.numpy(), tex.grad.numpy(), canvas[0].detach().cpu().numpy()


def fd(fn, x0, idx):
    out = []
    for k in idx:
        xp, xm = x0.astype(np.float64).copy(), x0.astype(np.float64).copy()
        xp.flat[k] += EPS
        xm.flat[k] -= EPS
        out.append((fn(xp), fn(xm)))
    return out


def test_phong_gradients_vs_fd64(cuda_device, scene):
    sc = scene
    flat_tex = np.full_like(sc.texture, 0.7)  # constant texels: no texel jumps under geometric moves
    base = oracle.render(phong_spec(sc, sc.eye, sc.light_direction, sc.position, flat_tex, np.float64),
                         np.ones((W, H)), np.ones((W, H, 3)), dtype=np.float64)
    target = base["canvas"] * 0.8 + 0.05
    rng = np.random.Generator(np.random.PCG64(7))
    visible = np.unique(base["prim_id"][base["prim_id"] >= 0])
    vert_idx = np.unique(sc.faces[rng.choice(visible, 4)].reshape(-1))[:6]
    cases = [("eye", k) for k in range(3)] + [("light", k) for k in range(3)] + [("pos", 3 * v + q) for v in vert_idx for q in (0, 2)]

    def render_with(kind, x):
        eye, light, pos = sc.eye, sc.light_direction, sc.position
        if kind == "eye":
            eye = x
        elif kind == "light":
            light = x
        else:
            pos = x.reshape(-1, 3)
        return oracle.render(phong_spec(sc, eye, light, pos, flat_tex, np.float64), np.ones((W, H)),
                             np.ones((W, H, 3)), dtype=np.float64)

    for kind, k in cases:
        x0 = {"eye": sc.eye, "light": sc.light_direction, "pos": sc.position.reshape(-1)}[kind].astype(np.float64)
        xp, xm = x0.copy(), x0.copy()
        xp[k] += EPS
        xm[k] -= EPS
        op, om = render_with(kind, xp), render_with(kind, xm)
        mask = ((op["prim_id"] == base["prim_id"]) & (om["prim_id"] == base["prim_id"]) & (base["prim_id"] >= 0)).astype(np.float64)
        lp = float((mask[..., None] * (op["canvas"] - target) ** 2).sum())
        lm = float((mask[..., None] * (om["canvas"] - target) ** 2).sum())
        g_fd = (lp - lm) / (2 * EPS)
        ge, gl, gp, _, _ = analytic(sc, mask, target, flat_tex, cuda_device)
        g_an = {"eye": ge, "light": gl, "pos": gp.reshape(-1)}[kind][k]
        scale = max(abs(g_fd), 1e-2)
        assert abs(g_an - g_fd) <= 2e-3 * scale + 1e-4, (kind, k, g_an, g_fd)


def test_texture_gradients_vs_fd64(cuda_device, scene):
    sc = scene
    spec64 = phong_spec(sc, sc.eye, sc.light_direction, sc.position, sc.texture, np.float64)
    base = oracle.render(spec64, np.ones((W, H)), np.ones((W, H, 3)), dtype=np.float64)
    target = base["canvas"] * 0.5
    mask = (base["prim_id"] >= 0).astype(np.float64)
    _, _, _, gt, _ = analytic(sc, mask, target, sc.texture, cuda_device)
    used = np.argwhere(np.abs(gt).sum(-1) > 0)[:5]
    assert len(used) >= 3
    for (u, v) in used:
        for ch in range(3):
            def loss(t):
                s = phong_spec(sc, sc.eye, sc.light_direction, sc.position, t, np.float64)
                return oracle_loss(s, target, mask)[0]
            tp, tm = sc.texture.astype(np.float64).copy(), sc.texture.astype(np.float64).copy()
            tp[u, v, ch] += EPS
            tm[u, v, ch] -= EPS
            g_fd = (loss(tp) - loss(tm)) / (2 * EPS)
            assert abs(gt[u, v, ch] - g_fd) <= 1e-3 * max(abs(g_fd), 1e-2) + 1e-5, (u, v, ch, gt[u, v, ch], g_fd)


def test_phong_reflection_shadow_light_terms_vs_fd64(cuda_device):
    flat = synthetic.brax_like_batch(2, seed=synthetic.BASE_SEED + 31)
    sb = jb.scene_batch_from_flat(flat, 64, 64, shadow_size=(96, 96), device=cuda_device)
    db = DifferentiableBatch(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0))
    names = ["ambient", "diffuse", "specular", "light_dir_eye", "light_colour"]
    leaves = {k: torch.tensor(np.asarray(sb.main_jobs[k], F32), requires_grad=True) for k in names}
    canvas, _ = db.render(**{k: v.to(cuda_device) for k, v in leaves.items()})
    target = torch.rand(canvas.shape, generator=torch.Generator().manual_seed(3)).to(cuda_device)
    ((canvas - target) ** 2).sum().backward()
    tgt = target.cpu().numpy().astype(np.float64)
    for s in range(2):
        dspec, mspec = jb.scene_job_specs(flat, sb, s)
        dref = oracle.render(dspec, np.full((96, 96), np.finfo(F32).max, F32))
        mspec.shadow_map = dref["zbuffer"]
        for name in names:
            for c in range(3):
                def loss(val):
                    setattr(mspec, name, val)
                    out = oracle.render(mspec, np.ones((64, 64)), np.ones((64, 64, 3)), dtype=np.float64)
                    return float(((out["canvas"] - tgt[s]) ** 2).sum())
                v0 = np.asarray(sb.main_jobs[name][s], np.float64)
                vp, vm = v0.copy(), v0.copy()
                vp[c] += EPS
                vm[c] -= EPS
                g_fd = (loss(vp) - loss(vm)) / (2 * EPS)
                setattr(mspec, name, v0)
                g_an = float(leaves[name].grad[s, c])
                assert abs(g_an - g_fd) <= 2e-3 * max(abs(g_fd), 1e-1) + 1e-3, (s, name, c, g_an, g_fd)


def test_depth_sum_gradient_wrt_world_to_clip(cuda_device):
    # tests/smoke_test_grad.py:92-107: grad of sum(depth) w.r.t. the camera
    from tests.scenes import random_job

    spec = random_job(_lib.SHADER_GOURAUD, seed=41, W=32, H=32, F=40, spread=1.0)
    spec.colour = np.abs(spec.colour)
    sb = jb.scene_batch_from_specs([spec], cuda_device)
    db = DifferentiableBatch(sb, form="plain")
    w2c = torch.tensor(spec.world_to_clip.astype(F32)[None], requires_grad=True)
    _, z = db.render(world_to_clip=w2c.to(cuda_device))
    base = oracle.render(spec, np.ones((32, 32)), np.ones((32, 32, 3)), dtype=np.float64)
    mask = torch.tensor(base["prim_id"] >= 0, device=cuda_device)
    (z[0] * mask).sum().backward()
    g = w2c.grad.numpy()[0]
    for (r, q) in [(0, 0), (1, 1), (2, 2), (2, 3), (3, 2), (0, 3)]:
        def loss(m):
            s2 = JobSpec(**{**spec.__dict__})
            s2.world_to_clip = m
            out = oracle.render(s2, np.ones((32, 32)), np.ones((32, 32, 3)), dtype=np.float64)
            keep = (out["prim_id"] == base["prim_id"]) & (base["prim_id"] >= 0)
            return float(out["zbuffer"][keep].sum()), keep
        mp, mm = spec.world_to_clip.astype(np.float64).copy(), spec.world_to_clip.astype(np.float64).copy()
        mp[r, q] += EPS
        mm[r, q] -= EPS
        lp, kp = loss(mp)
        lm, km = loss(mm)
        if (kp != (base["prim_id"] >= 0)).any() or (km != (base["prim_id"] >= 0)).any():
            continue  # visibility changed: not differentiable here
        g_fd = (lp - lm) / (2 * EPS)
        assert abs(g[r, q] - g_fd) <= 2e-3 * max(abs(g_fd), 1e-1) + 1e-3, (r, q, g[r, q], g_fd)


def _darboux_job():
    from tests.scenes import random_job

    spec = random_job(_lib.SHADER_PHONG_DARBOUX, seed=51, W=40, H=36, F=30, spread=1.0)
    spec.light_colour = np.ones(3, F32)
    spec.light_direction = np.array((0.2, -0.3, 0.93), F32)
    return spec


def _as64(spec):
    import copy

    s = copy.copy(spec)
    for name in ("position", "normal", "uv", "texture", "normal_map", "light_direction", "light_colour",
                 "viewport", "world_to_clip", "world_to_eye_norm"):
        setattr(s, name, np.asarray(getattr(spec, name), np.float64))
    return s


def test_phong_darboux_gradients_vs_fd64(cuda_device):
    """phong_darboux: gradients through the Darboux frame (vertex 0's NDC and
    uv triangles, the per-fragment 3x3 inverse), the normal map, the lighting
    and the interpolated normal, to positions, normals, normal-map and
    diffuse texels and the light direction."""
    spec = _darboux_job()
    Wd, Hd = spec.width, spec.height
    base = oracle.render(_as64(spec), np.ones((Wd, Hd)), np.ones((Wd, Hd, 3)), dtype=np.float64)
    assert (base["prim_id"] >= 0).sum() > 50
    target = base["canvas"] * 0.7 + 0.1
    sb = jb.scene_batch_from_specs([spec], cuda_device)
    db = DifferentiableBatch(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0))
    leaves = {
        "position": torch.tensor(spec.position, requires_grad=True),
        "normal": torch.tensor(spec.normal, requires_grad=True),
        "texture": torch.tensor(spec.texture.reshape(-1), requires_grad=True),
        "normal_map": torch.tensor(spec.normal_map.reshape(-1), requires_grad=True),
        "light_direction": torch.tensor(spec.light_direction[None], requires_grad=True),
    }

    def fd(name, flat_index, mutate):
        p, m = _as64(spec), _as64(spec)
        mutate(p, flat_index, EPS)
        mutate(m, flat_index, -EPS)
        op = oracle.render(p, np.ones((Wd, Hd)), np.ones((Wd, Hd, 3)), dtype=np.float64)
        om = oracle.render(m, np.ones((Wd, Hd)), np.ones((Wd, Hd, 3)), dtype=np.float64)
        mask = ((op["prim_id"] == base["prim_id"]) & (om["prim_id"] == base["prim_id"]) &
                (base["prim_id"] >= 0)).astype(np.float64)
        lp = float((mask[..., None] * (op["canvas"] - target) ** 2).sum())
        lm = float((mask[..., None] * (om["canvas"] - target) ** 2).sum())
        return (lp - lm) / (2 * EPS), mask

    def bump(field):
        def mutate(s, k, e):
            a = np.array(getattr(s, field), np.float64, copy=True)
            a.reshape(-1)[k] += e
            setattr(s, field, a)
        return mutate

    rng = np.random.Generator(np.random.PCG64(11))
    visible = np.unique(base["prim_id"][base["prim_id"] >= 0])
    verts = np.unique(spec.faces[rng.choice(visible, 3)].reshape(-1))[:4]
    cases = [("light_direction", k) for k in range(3)]
    cases += [("position", 3 * v + q) for v in verts for q in (0, 1)]
    cases += [("normal", 3 * v + q) for v in verts[:2] for q in range(3)]
    for name, k in cases:
        g_fd, mask = fd(name, k, bump(name))
        for t in leaves.values():
            t.grad = None
        canvas, _ = db.render(**{n: t.to(cuda_device) for n, t in leaves.items()})
        m = torch.tensor(mask, dtype=torch.float32, device=cuda_device)[None, ..., None]
        tg = torch.tensor(target, dtype=torch.float32, device=cuda_device)[None]
        (m * (canvas - tg) ** 2).sum().backward()
        g_an = float(leaves[name].grad.reshape(-1)[k])
        assert abs(g_an - g_fd) <= 3e-3 * max(abs(g_fd), 1e-2) + 2e-4, (name, k, g_an, g_fd)
    # texels of the normal map and of the diffuse texture that pixels sample
    mask = (base["prim_id"] >= 0).astype(np.float64)
    for t in leaves.values():
        t.grad = None
    canvas, _ = db.render(**{n: t.to(cuda_device) for n, t in leaves.items()})
    m = torch.tensor(mask, dtype=torch.float32, device=cuda_device)[None, ..., None]
    tg = torch.tensor(target, dtype=torch.float32, device=cuda_device)[None]
    (m * (canvas - tg) ** 2).sum().backward()
    for name, field in (("normal_map", "normal_map"), ("texture", "texture")):
        g = leaves[name].grad.numpy()
        used = np.argsort(-np.abs(g))[:4]
        assert np.abs(g[used]).min() > 0
        for k in used:
            def loss(e):
                s = _as64(spec)
                a = np.array(getattr(s, field), np.float64, copy=True)
                a.reshape(-1)[k] += e
                setattr(s, field, a)
                out = oracle.render(s, np.ones((Wd, Hd)), np.ones((Wd, Hd, 3)), dtype=np.float64)
                return float((mask[..., None] * (out["canvas"] - target) ** 2).sum())
            g_fd = (loss(EPS) - loss(-EPS)) / (2 * EPS)
            assert abs(g[k] - g_fd) <= 3e-3 * max(abs(g_fd), 1e-2) + 2e-4, (name, k, g[k], g_fd)


def test_specular_exponents_below_one_give_finite_gradients(cuda_device):
    # pow's slope at 0 is infinite for exponents below 1; where the clamp
    # max(r_z, 0) is below its kink the gradient through it is exactly 0
    from tests.scenes import random_job

    spec = random_job(_lib.SHADER_PHONG_REFLECTION, seed=44, W=40, H=40, F=60, spread=1.2)
    spec.specular_map = np.full_like(spec.specular_map, 0.6)
    sb = jb.scene_batch_from_specs([spec], cuda_device)
    db = DifferentiableBatch(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0))
    leaves = {"light_dir_eye": torch.tensor(spec.light_dir_eye[None], requires_grad=True),
              "position": torch.tensor(spec.position, requires_grad=True),
              "specular_map": torch.tensor(spec.specular_map.reshape(-1), requires_grad=True)}
    canvas, _ = db.render(**{k: v.to(cuda_device) for k, v in leaves.items()})
    (canvas ** 2).sum().backward()
    for k, v in leaves.items():
        assert torch.isfinite(v.grad).all(), k
    assert leaves["light_dir_eye"].grad.abs().sum() > 0
