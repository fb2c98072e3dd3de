"""GPU parity of the compiled primitive_chooser / mix hooks: the layered
chooser with the nearest and "over" mixers, plain and tiled forms, against
the oracle; layered and default jobs in one batch; the entry points' refusals
(tile shapes without a layered variant, the backward)."""
import ctypes

import numpy as np
import pytest
import torch

from jaxrenderer_gb300 import _lib, hooks, pipeline
from jaxrenderer_gb300.jobs import pack, render_plain, render_tiled, unpack
from jaxrenderer_gb300.shaders import PhongReflectionTextureShader
from jaxrenderer_gb300.types import Buffers, LightSource
from oracle import oracle
from tests import scenes
from tests.test_gpu_plain import assert_parity

pytestmark = pytest.mark.gpu
F32 = np.float32
LAYERED_SHADERS = [s for s in scenes.ALL_SHADERS if s != _lib.SHADER_DEPTH]
LAYERED_TILES = [(8, 8), (16, 8), (8, 4), (4, 8), (16, 16, 2), (8, 16, 2), (8, 8, 2)]  # (w, h[, warps per tile])


def layered_job(shader, seed, layers, mixer, opacity=0.5, F=90):
    spec = scenes.random_job(shader, seed=seed, F=F, spread=1.0)
    spec.layers, spec.mixer = layers, mixer
    spec.background = (0.2, 0.4, 0.6)
    if opacity == "per_face":
        rng = np.random.Generator(np.random.PCG64(seed))
        spec.face_alpha = rng.uniform(0.05, 0.95, spec.n_faces).astype(F32)
    else:
        spec.opacity = opacity
    return spec


def _render(specs, device, form, tile=(8, 8), count_ties=True):
    bufs = [scenes.initial_buffers(s) for s in specs]
    packed = pack(specs, [b[0] for b in bufs], [b[1] for b in bufs], device, count_ties=count_ties)
    if form == "plain":
        render_plain(packed)
    else:
        assert render_tiled(packed, tile=tile[:2], warps_per_tile=tile[2] if len(tile) > 2 else 1).overflow == 0
    outs = [tuple(t.clone() for t in o) for o in unpack(packed, specs)]
    ties = None if packed.near_ties is None else int(packed.near_ties.item())
    return outs, bufs, ties


@pytest.mark.parametrize("shader", LAYERED_SHADERS)
@pytest.mark.parametrize("layers,mixer,opacity", [(1, _lib.MIX_NEAREST, 1.0), (2, _lib.MIX_NEAREST, 1.0),
                                                  (3, _lib.MIX_OVER, 0.45), (4, _lib.MIX_OVER, "per_face")])
def test_layered_plain_and_tiled_match_oracle(cuda_device, shader, layers, mixer, opacity):
    spec = layered_job(shader, 300 + 10 * shader + layers, layers, mixer, opacity)
    if shader == _lib.SHADER_PHONG_REFLECTION_SHADOW:
        spec.shadow_map = np.random.default_rng(shader).uniform(0.2, 1.0, (24, 18)).astype(F32)
    plain, bufs, tp = _render([spec], cuda_device, "plain")
    ref = oracle.render(spec, *bufs[0])
    assert_parity(plain[0][0], plain[0][1], plain[0][2], ref, f"plain shader {shader} L={layers}")
    assert tp == ref["near_ties"]
    for tile in LAYERED_TILES:
        tiled, _, tt = _render([spec], cuda_device, "tiled", tile)
        for a, b in zip(tiled[0], plain[0]):
            if a.dtype == torch.float32:
                a, b = a.view(torch.int32), b.view(torch.int32)
            assert torch.equal(a, b), tile
        assert tt == tp
    assert (ref["prim_id"] >= 0).any()


def test_layered_and_default_jobs_in_one_batch(cuda_device):
    specs = []
    for k, shader in enumerate(LAYERED_SHADERS):
        s = scenes.random_job(shader, seed=500 + k, F=70 + 10 * k, spread=1.1)
        if k % 2 == 0:
            s.layers, s.mixer = 1 + k % _lib.MAX_LAYERS, _lib.MIX_OVER
            s.opacity, s.background = 0.3 + 0.1 * k, (1.0, 0.5, 0.0)
        if shader == _lib.SHADER_PHONG_REFLECTION_SHADOW:
            s.shadow_map = np.full((16, 16), 0.5, F32)
        specs.append(s)
    for form, tile in (("plain", None), ("tiled", (8, 8)), ("tiled", (16, 8))):
        outs, bufs, ties = _render(specs, cuda_device, form, tile or (8, 8), count_ties=False)
        for k, s in enumerate(specs):
            ref = oracle.render(s, *bufs[k])
            assert_parity(*outs[k], ref, f"{form} {tile} job {k}")


def test_hooked_shader_through_pipeline_render(cuda_device):
    class Glass(PhongReflectionTextureShader):
        primitive_chooser = hooks.LayeredChooser(4)
        mix = hooks.OverMixer(opacity=0.35, background=(0.9, 0.9, 1.0))

    spec = layered_job(_lib.SHADER_PHONG_REFLECTION, 77, 4, _lib.MIX_OVER, 0.35)
    spec.background = (0.9, 0.9, 1.0)
    z0, c0 = scenes.initial_buffers(spec)
    extra = PhongReflectionTextureShader.extra_input(
        position=spec.position, normal=spec.normal, uv=spec.uv,
        light=LightSource(direction=spec.light_direction, colour=spec.light_colour),
        light_dir_eye=spec.light_dir_eye, texture_shape=spec.texture_shape, texture_index=spec.texture_index,
        texture_offset=spec.texture_offset, texture=spec.texture, specular_map=spec.specular_map,
        ambient=spec.ambient, diffuse=spec.diffuse, specular=spec.specular)
    camera = scenes.perspective_camera(spec.width, spec.height)
    out, pid, _ = pipeline.render_with_ids(camera, Glass, Buffers(zbuffer=z0, targets=(c0,)), spec.faces, extra)
    ref = oracle.render(spec, z0, c0)
    assert_parity(out.zbuffer, out.targets[0], pid, ref, "pipeline.render with hooks")


def test_tile_shape_without_layered_variant_is_refused(cuda_device):
    spec = layered_job(_lib.SHADER_PHONG, 9, 2, _lib.MIX_NEAREST)
    z0, c0 = scenes.initial_buffers(spec)
    packed = pack([spec], [z0], [c0], cuda_device)
    with pytest.raises(RuntimeError, match="UNSUPPORTED"):
        render_tiled(packed, tile=(16, 16))


def test_backward_needs_the_saved_slots(cuda_device):
    spec = layered_job(_lib.SHADER_PHONG, 11, 2, _lib.MIX_OVER)
    z0, c0 = scenes.initial_buffers(spec)
    packed = pack([spec], [z0], [c0], cuda_device)
    assert packed.layer_prim is not None
    render_plain(packed)
    lib = _lib.load()
    b = packed.batch
    n = int(lib.rast_backward_workspace_bytes(ctypes.byref(b)))
    ws = torch.empty(max(n, 256), dtype=torch.uint8, device=cuda_device)
    gc = torch.zeros_like(packed.canvas)
    grads = _lib.RastGradPools()
    s = torch.cuda.current_stream(cuda_device).cuda_stream
    saved = b.pools.layer_prim
    b.pools.layer_prim = None
    st = lib.rast_backward(ctypes.byref(b), gc.data_ptr(), None, ctypes.byref(grads), ws.data_ptr(), n, s)
    assert _lib.STATUS_NAMES[st] == "RAST_ERR_INVALID_ARGUMENT"
    b.pools.layer_prim = saved
    st = lib.rast_backward(ctypes.byref(b), gc.data_ptr(), None, ctypes.byref(grads), ws.data_ptr(), n, s)
    assert st == 0
    # the saved slots: slot 0 is the nearest candidate; the shown primitive is
    # the first kept slot (phong keeps every candidate)
    lp = packed.layer_prim.reshape(_lib.MAX_LAYERS, -1)
    pid = packed.prim_id.reshape(-1)
    assert torch.equal(lp[0], pid)
    assert (lp[2:] == -1).all()  # layers = 2


def test_scene_batch_layers_tiled_equals_plain_and_oracle(cuda_device):
    from jaxrenderer_gb300 import batch as jb, synthetic

    n = 16
    inst = synthetic.brax_like_instances(n, seed=synthetic.BASE_SEED + 35)
    sb, _ = jb.scene_batch_from_instances(inst, 84, 84, shadow_size=(128, 128), device=cuda_device)
    opacity = np.linspace(0.2, 0.9, n).astype(F32)
    jb.set_layers(sb, 3, _lib.MIX_OVER, opacity=opacity, background=(0.5, 0.6, 0.7))
    runner = jb.BatchRunner(sb, form="tiled")
    runner.capture()
    got = runner.replay()
    got = {k: getattr(got, k).clone() for k in ("canvas", "zbuffer", "prim_id")}
    want = jb.BatchRunner(sb, form="plain").run()
    for k, g in got.items():
        w = getattr(want, k)
        if g.dtype == torch.float32:
            g, w = g.view(torch.int32), w.view(torch.int32)
        assert torch.equal(g, w), k
    for s in (0, 9):
        sub = inst.host_flat([s])
        tables = jb.scene_batch_tables(sub, 84, 84, shadow_size=(128, 128))
        dspec, mspec = jb.scene_job_specs(sub, tables, 0)
        mspec.layers, mspec.mixer, mspec.opacity, mspec.background = 3, _lib.MIX_OVER, opacity[s], (0.5, 0.6, 0.7)
        dref = oracle.render(dspec, np.full((128, 128), np.finfo(F32).max, F32))
        mspec.shadow_map = dref["zbuffer"]
        ref = oracle.render(mspec, np.ones((84, 84), F32), np.ones((84, 84, 3), F32))
        assert_parity(got["zbuffer"][s], got["canvas"][s], got["prim_id"][s], ref, f"layered scene {s}")


def _over_job():
    spec = layered_job(_lib.SHADER_PHONG_REFLECTION, 61, 3, _lib.MIX_OVER, "per_face", F=50)
    spec.background = (0.3, 0.5, 0.7)
    return spec


def _spec64(spec):
    import copy

    s = copy.copy(spec)
    for name in ("position", "normal", "uv", "texture", "specular_map", "viewport", "world_to_clip",
                 "world_to_eye_norm", "light_dir_eye", "ambient", "diffuse", "specular", "light_colour"):
        setattr(s, name, np.asarray(getattr(spec, name), np.float64))
    s.background = np.asarray(spec.background, np.float64)
    s.face_alpha = np.asarray(spec.face_alpha, np.float64)
    return s


def test_over_mixer_gradients_vs_fd64(cuda_device):
    """The over mixer's backward (one pass per kept slot, weighted by its
    w = T a, and the background seen through T) against central differences
    of the FP64 oracle: texels, light and material terms, the background,
    and positions of faces shown in some slot (pixels whose slots change
    under the perturbation are masked out on both sides)."""
    from jaxrenderer_gb300 import batch as jb
    from jaxrenderer_gb300.autograd import DifferentiableBatch

    eps = 1e-3
    spec = _over_job()
    Wd, Hd = spec.width, spec.height
    z1, c1 = np.ones((Wd, Hd)), np.ones((Wd, Hd, 3))
    base = oracle.render(_spec64(spec), z1, c1, dtype=np.float64)
    assert (base["prim_id"] >= 0).sum() > 100
    target = base["canvas"] * 0.6 + 0.1
    sb = jb.scene_batch_from_specs([spec], cuda_device)
    db = DifferentiableBatch(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0))
    names = ["ambient", "diffuse", "specular", "light_dir_eye", "background"]
    leaves = {k: torch.tensor(np.asarray(getattr(spec, k), F32)[None], requires_grad=True) for k in names}
    leaves["texture"] = torch.tensor(spec.texture.reshape(-1), requires_grad=True)
    leaves["position"] = torch.tensor(spec.position, requires_grad=True)
    canvas, _ = db.render(**{k: v.to(cuda_device) for k, v in leaves.items()})
    layers0 = db.runner.layer_prim.clone()
    tgt = torch.tensor(target, dtype=torch.float32, device=cuda_device)[None]
    ((canvas - tgt) ** 2).sum().backward()

    def loss(s, mask=None):
        out = oracle.render(s, z1, c1, dtype=np.float64)
        d = (out["canvas"] - target) ** 2
        return float((d if mask is None else mask[..., None] * d).sum())

    # smooth parameters: no visibility change
    for name in names:
        for c in range(3):
            sp, sm = _spec64(spec), _spec64(spec)
            getattr(sp, name)[c] += eps
            getattr(sm, name)[c] -= eps
            g_fd = (loss(sp) - loss(sm)) / (2 * eps)
            g_an = float(leaves[name].grad[0, c])
            assert abs(g_an - g_fd) <= 2e-3 * max(abs(g_fd), 1e-1) + 1e-3, (name, c, g_an, g_fd)
    gt = leaves["texture"].grad.numpy().reshape(spec.texture.shape)
    used = np.argwhere(np.abs(gt).sum(-1) > 0)[:6]
    assert len(used) >= 3
    for (u, v) in used:
        for ch in range(3):
            sp, sm = _spec64(spec), _spec64(spec)
            sp.texture[u, v, ch] += eps
            sm.texture[u, v, ch] -= eps
            g_fd = (loss(sp) - loss(sm)) / (2 * eps)
            assert abs(gt[u, v, ch] - g_fd) <= 1e-3 * max(abs(g_fd), 1e-2) + 1e-5, (u, v, ch, gt[u, v, ch], g_fd)
    # positions: flat texture and specular maps (no texel jumps as corners
    # move) and slot-stable pixels only, judged by the GPU's saved slots
    gp = leaves["position"].grad.numpy()
    assert np.abs(gp).sum() > 0
    spec.texture = np.full_like(spec.texture, 0.8)
    spec.specular_map = np.full_like(spec.specular_map, 3.0)
    base = oracle.render(_spec64(spec), z1, c1, dtype=np.float64)
    target = base["canvas"] * 0.6 + 0.1
    tgt = torch.tensor(target, dtype=torch.float32, device=cuda_device)[None]
    db = DifferentiableBatch(jb.scene_batch_from_specs([spec], cuda_device), form="tiled",
                             tiled_config=_lib.RastTiledConfig(8, 8, 0))
    db.render()
    layers0 = db.runner.layer_prim.clone()
    rng = np.random.Generator(np.random.PCG64(3))
    shown = np.unique(layers0[layers0 >= 0].cpu().numpy())
    checked = 0
    for f in rng.choice(shown, size=min(6, len(shown)), replace=False):
        v = int(spec.faces[f][rng.integers(0, 3)])
        for q in (0, 1):
            pos_p, pos_m = spec.position.copy(), spec.position.copy()
            pos_p[v, q] += F32(eps)
            pos_m[v, q] -= F32(eps)
            stable = np.ones((Wd, Hd), bool)
            for pos in (pos_p, pos_m):
                db.render(position=torch.tensor(pos).to(cuda_device))
                lp = db.runner.layer_prim.reshape(_lib.MAX_LAYERS, Wd, Hd)
                stable &= (lp == layers0.reshape(_lib.MAX_LAYERS, Wd, Hd)).all(0).cpu().numpy()
            mask = stable.astype(np.float64)
            sp, sm = _spec64(spec), _spec64(spec)
            sp.position[v, q] += eps
            sm.position[v, q] -= eps
            g_fd = (loss(sp, mask) - loss(sm, mask)) / (2 * eps)
            # the analytic side with the same mask
            leaf = torch.tensor(spec.position, requires_grad=True)
            cv, _ = db.render(position=leaf.to(cuda_device))
            m = torch.tensor(mask, dtype=torch.float32, device=cuda_device)[None, ..., None]
            (m * (cv - tgt) ** 2).sum().backward()
            g_an = float(leaf.grad[v, q])
            assert abs(g_an - g_fd) <= 3e-3 * max(abs(g_fd), 1e-1) + 1e-3, (v, q, g_an, g_fd)
            checked += 1
    assert checked >= 6
