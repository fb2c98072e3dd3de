"""GPU parity of the plain form against the oracle, through the C ABI.

Bar: winning-primitive buffer and z-buffer bit-exact, colours within 1e-5
absolute (the specular power is the one operation whose CUDA and C library
results may differ by an ulp)."""
import numpy as np
import pytest
import torch

import jaxrenderer_gb300 as jr
from jaxrenderer_gb300 import _lib, batch as jb, synthetic
from jaxrenderer_gb300.jobs import JobSpec
from jaxrenderer_gb300.pipeline import render_job
from jaxrenderer_gb300.renderer import Renderer
from oracle import oracle
from tests import scenes

pytestmark = pytest.mark.gpu
F32 = np.float32
COLOUR_ATOL = 1e-5


def assert_parity(got_z, got_c, got_p, ref, what=""):
    gp = got_p.cpu().numpy()
    np.testing.assert_array_equal(gp, ref["prim_id"], err_msg=f"prim_id {what}")
    gz = got_z.cpu().numpy()
    np.testing.assert_array_equal(gz.view(np.uint32), ref["zbuffer"].view(np.uint32), err_msg=f"zbuffer {what}")
    if ref["canvas"] is not None:
        np.testing.assert_allclose(got_c.cpu().numpy(), ref["canvas"], atol=COLOUR_ATOL, rtol=0, err_msg=f"canvas {what}")


@pytest.mark.parametrize("shader", scenes.ALL_SHADERS)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_scene_parity(cuda_device, shader, seed):
    spec = scenes.random_job(shader, seed=100 * shader + seed, F=80 + 40 * seed, spread=1.2 + seed)
    z0, c0 = scenes.initial_buffers(spec)
    z, c, p, ties = render_job(spec, z0, c0, count_ties=True)
    ref = oracle.render(spec, z0, c0)
    assert_parity(z, c, p, ref, f"shader {shader} seed {seed}")
    assert int(ties.item()) == ref["near_ties"]
    assert (ref["prim_id"] >= 0).any()


@pytest.mark.parametrize("shader", [_lib.SHADER_DEPTH, _lib.SHADER_PHONG_REFLECTION])
def test_camera_inside_the_soup(cuda_device, shader):
    # eye among the triangles: primitives cross w = 0 (no clipping in the
    # reference), and primitives behind the eye must never win
    spec = scenes.random_job(shader, seed=7, F=200, spread=3.0, eye=(0.2, 0.1, 0.5))
    z0, c0 = scenes.initial_buffers(spec)
    z, c, p, _ = render_job(spec, z0, c0)
    assert_parity(z, c, p, oracle.render(spec, z0, c0), "inside")


def test_reference_smoke_batched_triangles(cuda_device):
    spec = scenes.smoke_batched_triangles_job()
    z0 = np.ones((1920, 1080), F32)
    c0 = np.zeros((1920, 1080, 3), F32)
    z, c, p, _ = render_job(spec, z0, c0)
    scenes.smoke_batched_triangles_asserts(z.cpu().numpy(), c.cpu().numpy())
    assert_parity(z, c, p, oracle.render(spec, z0, c0, n_threads=8), "smoke")


def test_config1_cube_get_camera_image(cuda_device):
    W, H = 640, 480
    cube = jr.create_cube(np.ones(3, F32), np.ones(2, F32),
                          np.zeros((2, 2, 3), F32) + np.array([0, 0, 1], F32), np.ones((2, 2), F32) * 2.0)
    params = jr.CameraParameters(viewWidth=W, viewHeight=H, position=np.array([2.0, 4.0, 1.0], F32))
    objects = [jr.ModelObject(model=cube)]
    image = Renderer.get_camera_image(objects=objects, camera=params, light=jr.LightParameters(), width=W, height=H)
    cam = Renderer.create_camera_from_parameters(params)
    extra, fi = Renderer._extra(jr.merge_objects(objects), jr.LightParameters(), cam)
    spec = jr.jobs.job_from_extra(_lib.SHADER_PHONG_REFLECTION, cam, extra, W, H)
    spec.faces = fi
    ref = oracle.render(spec, np.ones((W, H), F32), np.ones((W, H, 3), F32), n_threads=8)
    np.testing.assert_allclose(image.cpu().numpy(), ref["canvas"], atol=COLOUR_ATOL, rtol=0)
    assert set(np.unique(ref["prim_id"])) == {-1, 6, 7, 10, 11}


def test_renderer_with_shadow_pass(cuda_device):
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 5))
    scene = synthetic.brax_like_scene(rng)
    W = H = 84
    params = jr.CameraParameters(viewWidth=W, viewHeight=H, position=scene.camera_position, hfov=58.0, vfov=58.0)
    cam = Renderer.create_camera_from_parameters(params)
    model = jr.merge_objects(scene.objects)
    light = jr.LightParameters()
    sp = jr.ShadowParameters()
    buffers = Renderer.create_buffers(W, H)
    out, ids = Renderer.render(model, light, cam, buffers, shadow_param=sp, with_ids=True)
    # oracle chain: depth pass into a float32-max map (+offset), then main pass
    shadow_cam = jr.Shadow.light_camera(np.asarray(light.direction, F32), cam.viewport, sp.centre, sp.up)
    depth = JobSpec(shader=_lib.SHADER_DEPTH, width=W, height=H, viewport=shadow_cam.viewport,
                    world_to_clip=shadow_cam.world_to_clip, world_to_eye_norm=shadow_cam.world_to_eye_norm,
                    position=np.asarray(model.verts, F32), faces=np.asarray(model.faces, np.int32),
                    depth_offset=sp.offset, apply_depth_offset=True)
    smap = oracle.render(depth, np.full((W, H), np.finfo(F32).max, F32))["zbuffer"]
    extra, fi = Renderer._extra(model, light, cam)
    shadow = jr.Shadow(shadow_map=smap, strength=sp.strength, camera=shadow_cam)
    from jaxrenderer_gb300.shaders import PhongReflectionShadowTextureExtraInput
    ex = PhongReflectionShadowTextureExtraInput(**extra._asdict(), shadow=shadow, camera=cam)
    spec = jr.jobs.job_from_extra(_lib.SHADER_PHONG_REFLECTION_SHADOW, cam, ex, W, H)
    spec.faces = fi
    ref = oracle.render(spec, np.ones((W, H), F32), np.ones((W, H, 3), F32))
    assert_parity(out.zbuffer, out.targets[0], ids, ref, "renderer+shadow")


def test_batch_of_uneven_scenes_matches_per_scene_oracle(cuda_device):
    flat = synthetic.brax_like_batch(6, seed=synthetic.BASE_SEED + 9)
    sb = jb.scene_batch_from_flat(flat, 84, 84, shadow_size=(128, 128), device=cuda_device)
    out = jb.BatchRunner(sb, form="plain").run()
    torch.cuda.synchronize()
    for s in range(sb.n_scenes):
        dspec, mspec = scenes.specs_from_batch(flat, sb, s)
        dref = oracle.render(dspec, np.full((128, 128), np.finfo(F32).max, F32))
        np.testing.assert_array_equal(out.shadow_prim_id[s].cpu().numpy(), dref["prim_id"])
        np.testing.assert_array_equal(out.shadow_map[s].cpu().numpy().view(np.uint32), dref["zbuffer"].view(np.uint32))
        mspec.shadow_map = dref["zbuffer"]
        ref = oracle.render(mspec, np.ones((84, 84), F32), np.ones((84, 84, 3), F32))
        assert_parity(out.zbuffer[s], out.canvas[s], out.prim_id[s], ref, f"scene {s}")


def test_mixed_shader_job_batch(cuda_device):
    specs = [scenes.random_job(sh, seed=500 + sh, W=24 + 4 * sh, H=20 + 3 * sh, F=30 + 10 * sh)
             for sh in scenes.ALL_SHADERS]
    bufs = [scenes.initial_buffers(s) for s in specs]
    packed = jr.jobs.pack(specs, [b[0] for b in bufs], [b[1] for b in bufs], cuda_device)
    jr.jobs.render_plain(packed)
    for s, (z, c, p), (z0, c0) in zip(specs, jr.jobs.unpack(packed, specs), bufs):
        assert_parity(z, c if c0 is not None else None, p, oracle.render(s, z0, c0), f"shader {s.shader}")


def test_empty_face_list_leaves_buffers(cuda_device):
    spec = scenes.random_job(_lib.SHADER_GOURAUD, seed=3)
    spec.faces = np.zeros((0, 3), np.int32)
    z0, c0 = scenes.initial_buffers(spec, zdefault=0.25, cdefault=(0.1, 0.2, 0.3))
    z, c, p, _ = render_job(spec, z0, c0)
    np.testing.assert_array_equal(z.cpu().numpy(), z0)
    np.testing.assert_array_equal(c.cpu().numpy(), c0)
    assert (p.cpu().numpy() == -1).all()
