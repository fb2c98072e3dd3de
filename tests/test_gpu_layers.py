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
LAYERED_TILES = [(8, 8), (16, 8), (8, 4), (4, 8)]


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
        assert render_tiled(packed, tile=tile).overflow == 0
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


def test_backward_refuses_layered_batches(cuda_device):
    spec = layered_job(_lib.SHADER_PHONG, 11, 2, _lib.MIX_NEAREST)
    z0, c0 = scenes.initial_buffers(spec)
    packed = pack([spec], [z0], [c0], cuda_device)
    render_plain(packed)
    lib = _lib.load()
    b = packed.batch
    n = int(lib.rast_backward_workspace_bytes(ctypes.byref(b)))
    ws = torch.empty(max(n, 256), dtype=torch.uint8, device=cuda_device)
    gc = torch.zeros_like(packed.canvas)
    grads = _lib.RastGradPools()
    st = lib.rast_backward(ctypes.byref(b), gc.data_ptr(), None, ctypes.byref(grads), ws.data_ptr(), n,
                           torch.cuda.current_stream(cuda_device).cuda_stream)
    assert _lib.STATUS_NAMES[st] == "RAST_ERR_UNSUPPORTED"


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
