"""CPU tests of the host-side mirror of the reference API."""
import numpy as np
import pytest

import jaxrenderer_gb300 as jr
from jaxrenderer_gb300 import synthetic
from jaxrenderer_gb300.renderer import Renderer, gather_rows
from jaxrenderer_gb300.utils import transpose_for_display

F32 = np.float32
SHAPES = [(1, 1), (1, 7), (3, 1), (20, 31, 3), (11, 11, 4)]


# tests/test_utils.py:18-128 of the reference, on NumPy arrays
@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("flip_vertical", [True, False])
def test_transpose_for_display_shape(shape, flip_vertical):
    m = np.random.Generator(np.random.PCG64(20230701)).uniform(size=shape)
    t = transpose_for_display(m, flip_vertical=flip_vertical)
    assert m.shape == shape
    assert t.shape == (shape[1], shape[0], *shape[2:])
    u1, c1 = np.unique(m, return_counts=True)
    u2, c2 = np.unique(t, return_counts=True)
    np.testing.assert_array_equal(u1, u2)
    np.testing.assert_array_equal(c1, c2)


@pytest.mark.parametrize("shape", SHAPES)
def test_transpose_for_display_flip(shape):
    m = np.random.Generator(np.random.PCG64(20230701)).uniform(size=shape)
    a = transpose_for_display(m, flip_vertical=True)
    b = transpose_for_display(m, flip_vertical=False)
    np.testing.assert_array_equal(a, b[::-1])
    np.testing.assert_array_equal(b, np.swapaxes(m, 0, 1))


def test_camera_matrices_close_to_float64():
    p = jr.CameraParameters(viewWidth=640, viewHeight=480, position=np.array((2.0, 4.0, 1.0), F32))
    cam = Renderer.create_camera_from_parameters(p)
    eye = np.array((2.0, 4.0, 1.0))
    f = -eye / np.linalg.norm(eye)
    s = np.cross(f, (0, 0, 1.0))
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    view = np.identity(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    t = np.identity(4)
    t[:3, 3] = -eye
    view = view @ t
    fy = 1 / np.tan(np.radians(45.0) / 2)
    aspect = np.tan(np.radians(58.0) / 2) / np.tan(np.radians(45.0) / 2)
    proj = np.zeros((4, 4))
    proj[0, 0], proj[1, 1] = fy / aspect, fy
    proj[2, 2] = (1000 + 0.01) / (0.01 - 1000)
    proj[2, 3] = 2 * 1000 * 0.01 / (0.01 - 1000)
    proj[3, 2] = -1
    np.testing.assert_allclose(cam.world_to_clip, proj @ view, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(cam.view_inv @ cam.view, np.identity(4), atol=1e-5)
    vp = cam.viewport
    assert vp[0, 0] == 320 and vp[1, 1] == 240 and vp[0, 3] == 320 and vp[2, 2] == 0.5


def test_merge_objects_offsets_and_maps():
    a = jr.create_cube(np.ones(3, F32), np.ones(2, F32), np.ones((2, 3, 3), F32), np.ones((2, 3), F32))
    b = jr.create_capsule(0.5, 1.0, jr.UpAxis.Z, np.zeros((4, 2, 3), F32), np.zeros((4, 2), F32))
    t = np.identity(4, dtype=F32)
    t[:3, 3] = (1, 2, 3)
    m = jr.merge_objects([jr.ModelObject(model=a), jr.ModelObject(model=b, transform=t)])
    assert m.verts.shape == (24 + 576, 3)
    assert m.faces.max() == 24 + 576 - 1 and m.faces[12:].min() == 24
    assert m.diffuse_map.shape == (8, 3, 3) and m.offset == 4
    np.testing.assert_array_equal(m.texture_shape, [[2, 3], [4, 2]])
    lo, hi = m.verts[24:].min(axis=0), m.verts[24:].max(axis=0)
    np.testing.assert_allclose((lo + hi) / 2, (1, 2, 3), atol=1e-5)
    np.testing.assert_allclose(hi - lo, (1, 1, 3), atol=0.02)
    assert (m.texture_index[:24] == 0).all() and (m.texture_index[24:] == 1).all()


def test_gather_rows_clamps_like_jnp():
    a = np.arange(5)
    np.testing.assert_array_equal(gather_rows(a, [-1, -5, -6, 0, 4, 5, 9]), [4, 0, 0, 0, 4, 4, 4])


def test_shapes_counts():
    c = jr.create_cube(np.ones(3, F32), np.ones(2, F32), np.ones((2, 2, 3), F32), np.ones((2, 2), F32))
    assert c.verts.shape == (24, 3) and c.faces.shape == (12, 3)
    k = jr.create_capsule(1.0, 0.5, jr.UpAxis.Y, np.ones((1, 1, 3), F32), np.ones((1, 1), F32))
    assert k.verts.shape == (576, 3) and k.faces.shape == (192, 3)
    assert synthetic.icosphere(2)[1].shape == (320, 3)
    assert synthetic.icosphere(4)[1].shape == (5120, 3)
    assert synthetic.capsule_mesh(16, 8)[1].shape == (512, 3)


def test_brax_like_scene_sizes():
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 1))
    sizes = [synthetic.brax_like_scene(rng).n_faces for _ in range(20)]
    assert 2 + 8 * 12 <= min(sizes) and max(sizes) <= 2 + 32 * 512


def test_create_capsule_reproduces_the_reference_fixture_capsules():
    """The 17 capsules of the reference's Brax Ant inputs (tests/golden/
    brax_ant_30.npz, made by the reference's create_capsule from its
    tabulated sphere) come out of create_capsule bit for bit."""
    from pathlib import Path

    from jaxrenderer_gb300 import brax

    objects, _, _ = brax.load_batched_npz(Path(__file__).resolve().parent / "golden" / "brax_ant_30.npz")
    r8, h1, h2 = F32(0.08), F32(0.1414213627576828), F32(0.2828427255153656)
    params = [(F32(0.25), F32(0))] + [(r8, h) for h in (h1, h1, h1, h1, h1, h2, 0, h1, h2, 0, h1, h2, 0, h1, h2, 0)]
    for o, (radius, hh) in zip(objects[1:], params):
        m = o.model
        k = jr.create_capsule(radius, hh, jr.UpAxis.Z, np.asarray(m.diffuse_map)[0], np.asarray(m.specular_map)[0])
        for field in ("verts", "norms", "uvs", "faces", "faces_norm", "faces_uv"):
            np.testing.assert_array_equal(getattr(k, field), np.asarray(getattr(m, field))[0], err_msg=field)


def test_batched_camera_setup_matches_the_per_scene_setup_bitwise():
    """batch._cameras / _light_cameras (one camera per scene, vectorised)
    give each scene the bits Renderer.create_camera_from_parameters and
    Shadow.light_camera give it alone."""
    from jaxrenderer_gb300 import batch as jb
    from jaxrenderer_gb300.geometry import Camera, apply_vec_rows
    from jaxrenderer_gb300.shadow import Shadow

    rng = np.random.default_rng(5)
    pos = (rng.normal(size=(24, 3)) * 6).astype(F32)
    tgt = rng.normal(size=(24, 3)).astype(F32)
    params = jr.CameraParameters(viewWidth=96, viewHeight=64, hfov=58.0, vfov=32.625)
    w2c, w2e, view, vp = jb._cameras(pos, params, tgt)
    d = np.array((0.57735, -0.57735, 0.57735), F32)
    up = np.array((0, 0, 1), F32)
    sw, se = jb._light_cameras(d, vp, tgt, up)
    ldir = apply_vec_rows(d, view)
    for k in range(24):
        cam = jr.Renderer.create_camera_from_parameters(params._replace(position=pos[k], target=tgt[k]))
        light = Shadow.light_camera(d, vp, tgt[k], up)
        for got, want in ((w2c[k], cam.world_to_clip), (w2e[k], cam.world_to_eye_norm), (view[k], cam.view),
                          (sw[k], light.world_to_clip), (se[k], light.world_to_eye_norm),
                          (ldir[k], Camera.apply_vec(d, cam.view))):
            np.testing.assert_array_equal(got.view(np.uint32), np.asarray(want, F32).view(np.uint32))


def test_batch_axis_detection_and_frame_selection():
    """Renderer._batch_size / _take: a field with one more leading axis than
    the reference's NamedTuple gives it is a batch (jax.vmap of the call)."""
    from pathlib import Path

    from jaxrenderer_gb300 import brax

    objects, camera, target = brax.load_batched_npz(Path(__file__).resolve().parent / "golden" / "brax_ant_2.npz")
    R = jr.Renderer
    assert R._batch_size(objects) == 2 and R._batch_size(camera) == 2
    assert R._batch_size(jr.LightParameters(), jr.ShadowParameters()) is None
    assert R._batch_size(jr.ShadowParameters(centre=target)) == 2
    one = R._take(list(objects), 1)
    np.testing.assert_array_equal(one[3].transform, np.asarray(objects[3].transform)[1])
    assert np.shape(one[3].model.verts) == (576, 3)
    cam = R._take(camera, 1)
    np.testing.assert_array_equal(cam.position, np.asarray(camera.position)[1])
    assert int(cam.viewWidth) == 960
    with pytest.raises(ValueError):
        R._batch_size(camera, jr.ShadowParameters(centre=np.zeros((3, 3), F32)))


def test_frame_matrices_refresh_equals_a_full_table_build():
    """batch.frame_matrices (the per-call update of the batched
    get_camera_image path) writes what scene_batch_tables builds."""
    from pathlib import Path

    from jaxrenderer_gb300 import batch as jb, brax

    objects, camera, target = brax.load_batched_npz(Path(__file__).resolve().parent / "golden" / "brax_ant_30.npz")
    bb = brax.scenes_from_batched(objects, camera, target)
    shell = bb.scenes.shell()
    t = jb.scene_batch_tables(shell, 84, 84, bb.light, bb.shadow, (84, 84), bb.camera, shadow_viewport="camera")
    order = np.arange(30)[::-1].copy()
    shell.camera_position, shell.camera_target = shell.camera_position[order], shell.camera_target[order]
    moved = bb.shadow._replace(centre=bb.shadow.centre[order])
    want = jb.scene_batch_tables(shell, 84, 84, bb.light, moved, (84, 84), bb.camera, shadow_viewport="camera")
    jb.frame_matrices(t, shell.camera_position, shell.camera_target, bb.camera, bb.light, moved)
    assert t.main_jobs.tobytes() == want.main_jobs.tobytes()
    assert t.shadow_jobs.tobytes() == want.shadow_jobs.tobytes()


def test_dispatch_sends_canvases_wider_than_the_tiled_rectangles_to_the_plain_form():
    from types import SimpleNamespace

    from jaxrenderer_gb300 import dispatch

    def batch(w, h, f):
        return SimpleNamespace(jobs=[SimpleNamespace(width=w, height=h, n_faces=f)])

    assert dispatch.choose(batch(2048, 2048, 100_000), "auto") == "tiled"
    assert dispatch.choose(batch(70_000, 4, 1_000_000), "auto") == "plain"  # 16-bit pixel rectangles
    assert dispatch.choose(batch(84, 84, 10), "auto") == "plain"  # small pass: fewer launches
