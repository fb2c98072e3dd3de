"""The reference-facing API on the GPU: Renderer.get_camera_image and
Renderer.render with batched inputs (a leading axis of frames, the
jax.vmap use of the reference's notebooks and examples/batch_rendering.py),
against per-frame oracle renders, and the form each call picks (plain or
tiled, identical canvases either way)."""
import os
from pathlib import Path

import numpy as np
import pytest

import jaxrenderer_gb300 as jr
from jaxrenderer_gb300 import batched_api, brax, dispatch
from oracle import oracle

pytestmark = pytest.mark.gpu
F32 = np.float32
GOLDEN = Path(__file__).resolve().parent / "golden"
THREADS = max(1, len(os.sched_getaffinity(0)))
ATOL = 1e-5


def notebook_light():
    return jr.LightParameters(direction=np.array((0.57735, -0.57735, 0.57735), F32), ambient=np.full(3, 0.8, F32),
                              diffuse=np.full(3, 0.8, F32), specular=np.full(3, 0.6, F32))


def oracle_frame(objects, light, camera, W, H, shadow_param):
    """The host path of Renderer.render for one frame: merge_objects, the
    camera matrices, the depth pass, then the shadowed phong pass."""
    cam = jr.Renderer.create_camera_from_parameters(camera)
    model = jr.merge_objects(objects)
    depth, main = jr.Renderer._scene_specs(model, light, cam, W, H, shadow_param)
    if depth is not None:
        main.shadow_map = oracle.render(depth, np.full((W, H), np.finfo(F32).max, F32), n_threads=THREADS)["zbuffer"]
    return oracle.render(main, np.ones((W, H), F32), np.ones((W, H, 3), F32), n_threads=THREADS)


def frame_args(objects, camera, target, f):
    objs = jr.Renderer._take(list(objects), f)
    return objs, jr.Renderer._take(camera, f), jr.ShadowParameters(centre=np.asarray(target, F32)[f])


@pytest.mark.parametrize("W,H", [(84, 84), (320, 180)])
def test_batched_get_camera_image_on_the_brax_fixture_matches_oracle(cuda_device, W, H):
    objects, camera, target = brax.load_batched_npz(GOLDEN / "brax_ant_30.npz")
    light = notebook_light()
    shadow = jr.ShadowParameters(centre=target)
    img = jr.Renderer.get_camera_image(objects, light, camera, W, H, shadow_param=shadow)
    assert img.shape == (30, W, H, 3)
    for f in (0, 11, 29):
        objs, cam, sp = frame_args(objects, camera, target, f)
        ref = oracle_frame(objs, light, cam, W, H, sp)
        np.testing.assert_allclose(img[f].cpu().numpy(), ref["canvas"], rtol=0, atol=ATOL, err_msg=f"frame {f}")
        single = jr.Renderer.get_camera_image(objs, light, cam, W, H, shadow_param=sp)  # unbatched call
        np.testing.assert_allclose(single.cpu().numpy(), ref["canvas"], rtol=0, atol=ATOL)
    # second call, same meshes, frames in another order: the cached set-up takes the new placements
    order = np.arange(30)[::-1].copy()
    moved = [o._replace(transform=np.asarray(o.transform)[order], local_scaling=np.asarray(o.local_scaling)[order])
             for o in objects]
    camera2 = camera._replace(position=np.asarray(camera.position)[order], target=np.asarray(camera.target)[order])
    img2 = jr.Renderer.get_camera_image(moved, light, camera2, W, H,
                                        shadow_param=jr.ShadowParameters(centre=target[order]))
    for k in (0, 18):
        np.testing.assert_array_equal(img2[k].cpu().numpy(), img[order[k]].cpu().numpy())


def test_batched_paths_and_forms_agree(cuda_device):
    objects, camera, target = brax.load_batched_npz(GOLDEN / "brax_ant_2.npz")
    light = notebook_light()
    shadow = jr.ShadowParameters(centre=target)
    outs = []
    for form in ("plain", "tiled"):
        dispatch.set_render_form(form)
        try:
            outs.append(jr.Renderer.get_camera_image(objects, light, camera, 96, 64, shadow_param=shadow))
            # a light per frame takes the per-frame host merge path
            light_b = light._replace(colour=np.ones((2, 3), F32))
            outs.append(jr.Renderer.get_camera_image(objects, light_b, camera, 96, 64, shadow_param=shadow))
        finally:
            dispatch.set_render_form("auto")
    for o in outs[1:]:
        np.testing.assert_array_equal(o.cpu().numpy(), outs[0].cpu().numpy())


def test_batched_renderer_render_as_examples_batch_rendering(cuda_device):
    """examples/batch_rendering.py: 12 rotated capsules, merge_objects per
    object, batch_models, batched buffers, one Renderer.render over all."""
    tex = (np.array(((255, 255, 255), (255, 0, 0), (0, 255, 0), (0, 0, 255)), F32).reshape(2, 2, 3)[:, ::-1, :]
           / F32(255.0))
    cap = jr.create_capsule(0.1, 0.4, jr.UpAxis.Z, tex, np.full((2, 2), 2.0, F32))
    models = []
    for i in range(12):
        t = np.identity(4, F32)
        a = np.radians(30.0 * (i - 6))
        t[:3, :3] = np.array(((np.cos(a), 0, np.sin(a)), (0, 1, 0), (-np.sin(a), 0, np.cos(a))), F32)
        models.append(jr.merge_objects([jr.ModelObject(model=cap, transform=t)]))
    W, H = 160, 120
    camera = jr.Renderer.create_camera_from_parameters(
        jr.CameraParameters(viewWidth=W, viewHeight=H, position=np.array((0.0, 4.0, 0.0), F32),
                            target=np.zeros(3, F32)))
    light, shadow = jr.LightParameters(), jr.ShadowParameters()
    buffers = jr.Renderer.create_buffers(W, H, 12)
    out, ids = jr.Renderer.render(jr.batch_models(models), light, camera, buffers, shadow_param=shadow, with_ids=True)
    assert out.targets[0].shape == (12, W, H, 3) and ids.shape == (12, W, H)
    for i in (0, 5, 11):
        depth, main = jr.Renderer._scene_specs(models[i], light, camera, W, H, shadow)
        main.shadow_map = oracle.render(depth, np.full((W, H), np.finfo(F32).max, F32))["zbuffer"]
        ref = oracle.render(main, np.ones((W, H), F32), np.ones((W, H, 3), F32))
        np.testing.assert_array_equal(ids[i].cpu().numpy(), ref["prim_id"])
        np.testing.assert_array_equal(out.zbuffer[i].cpu().numpy().view(np.uint32), ref["zbuffer"].view(np.uint32))
        np.testing.assert_allclose(out.targets[0][i].cpu().numpy(), ref["canvas"], rtol=0, atol=ATOL)
        assert (ref["prim_id"] >= 0).sum() > 100


def test_auto_form_takes_the_tiled_form_for_large_passes(cuda_device):
    spec_small = jr.Renderer._scene_specs(jr.merge_objects([jr.ModelObject(model=jr.create_cube(
        np.ones(3, F32), np.ones(2, F32), np.ones((2, 2, 3), F32), np.ones((2, 2), F32)))]), jr.LightParameters(),
        jr.Renderer.create_camera_from_parameters(jr.CameraParameters(viewWidth=64, viewHeight=48,
                                                                      position=np.array((2.0, 4.0, 1.0), F32))),
        64, 48, None)[1]
    from jaxrenderer_gb300.jobs import pack

    small = pack([spec_small], [np.ones((64, 48), F32)], [np.ones((64, 48, 3), F32)], cuda_device)
    assert dispatch.choose(small) == "plain"
    n = 4000
    big = pack([spec_small] * n, [np.ones((64, 48), F32)] * n, [None] * n, cuda_device)
    assert dispatch.pass_pairs(big) >= dispatch.TILED_MIN_PAIRS and dispatch.choose(big) == "tiled"
    assert len(batched_api._CACHE) <= batched_api.MAX_CACHED
