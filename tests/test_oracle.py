"""CPU tests of the oracle (the C restatement): the reference's own smoke-test
assertions, known answers of its building blocks, and the tie/fallback rules."""
import numpy as np
import pytest

from jaxrenderer_gb300 import _lib
from jaxrenderer_gb300.geometry import Camera, det3, lu_inverse
from jaxrenderer_gb300.jobs import JobSpec
from oracle import oracle
from tests import scenes

F32 = np.float32


def test_reference_smoke_batched_triangles():
    spec = scenes.smoke_batched_triangles_job()
    z0 = np.full((1920, 1080), 1.0, F32)
    c0 = np.zeros((1920, 1080, 3), F32)
    out = oracle.render(spec, z0, c0, n_threads=8)
    scenes.smoke_batched_triangles_asserts(out["zbuffer"], out["canvas"])


def test_reference_smoke_perspective_geometry():
    # tests/smoke_test.py:233-329 with the built-in Gouraud shader standing in
    # for the test's custom checkerboard shader (depth does not depend on it).
    W, H = 1920, 1080
    cam = Camera.create(
        view=Camera.view_matrix(np.array((0.0, 0, 1), F32), np.zeros(3, F32), np.array((0.0, 1, 0), F32)),
        projection=Camera.perspective_projection_matrix(90.0, 1.0, -1.0, 1.0),
        viewport=Camera.viewport_matrix(np.zeros(2, np.int32), np.array((W, H)), 255),
    )
    pos = np.array(((-1.0, -1.0, -2.0), (1.0, -1.0, -1.0), (0.0, 1.0, -1.0)), F32)
    light = np.array((0.0, 0.0, -1.0), F32)
    spec = JobSpec(shader=_lib.SHADER_GOURAUD, width=W, height=H, viewport=cam.viewport,
                   world_to_clip=cam.world_to_clip, world_to_eye_norm=cam.world_to_eye_norm,
                   position=pos, faces=np.array(((0, 1, 2),), np.int32))
    spec.colour = np.eye(3, dtype=F32)
    spec.normal = np.tile(light, (3, 1))
    spec.light_direction = light
    out = oracle.render(spec, np.ones((W, H), F32), np.zeros((W, H, 3), F32), n_threads=8)
    z = out["zbuffer"].T[::-1]
    c = out["canvas"].transpose(1, 0, 2)[::-1]
    assert np.sum(z == 1.0) > (W * H // 2)
    assert z[679, 701] < z[779, 1388]
    empty = (c == 0).all(axis=2).sum()
    assert (W * H // 2) < empty < W * H


def test_inverse_and_det_known_answers():
    rng = np.random.Generator(np.random.PCG64(1))
    for _ in range(200):
        m = rng.normal(size=(3, 3)).astype(F32)
        inv = oracle.inv3(m)
        np.testing.assert_allclose(inv, np.linalg.inv(m.astype(np.float64)), rtol=2e-3, atol=2e-4)
        np.testing.assert_allclose(oracle.det3(m), np.linalg.det(m.astype(np.float64)), rtol=1e-4, atol=1e-5)


def test_host_restatement_matches_oracle_bitwise():
    # the host LU inverse (used for camera/model matrices) and the oracle's
    # are two restatements of the same algorithm: identical bits
    rng = np.random.Generator(np.random.PCG64(2))
    ms = rng.normal(size=(300, 3, 3)).astype(F32)
    ms[0] = np.array([[0, 1, 2], [3, 0, 5], [6, 7, 0]], F32)  # zero pivots force swaps
    ms[1] = np.array([[1e-30, 1, 0], [1, 1, 0], [0, 0, 1]], F32)  # subnormal-scale pivot
    host = lu_inverse(ms)
    for k in range(len(ms)):
        np.testing.assert_array_equal(host[k].view(np.uint32), oracle.inv3(ms[k]).view(np.uint32))
        assert det3(ms[k]).view(np.uint32) == oracle.det3(ms[k]).view(np.uint32)


def test_depth_order_is_monotone():
    zs = np.array([-np.inf, -1e30, -2.0, -1e-40, -0.0, 0.0, 1e-40, 0.5, 1.0, 3e38, np.inf], F32)
    o = [oracle.depth_order(z) for z in zs]
    assert all(a <= b for a, b in zip(o, o[1:]))
    assert oracle.depth_order(-0.0) == oracle.depth_order(0.0)
    assert oracle.depth_order(np.nan) == 0


def _two_triangle_job(shader, second_offset=0.0, flip_first=False):
    W, H = 16, 16
    cam = scenes.perspective_camera(W, H, eye=(0.0, 0.0, 3.0))
    tri = np.array([(-1, -1, 0), (1, -1, 0), (0, 1, 0)], F32)
    t0 = tri[[0, 2, 1]] if flip_first else tri
    t1 = tri + np.array([0, 0, second_offset], F32)
    verts = np.concatenate([t0, t1])
    spec = JobSpec(shader=shader, width=W, height=H, viewport=cam.viewport, world_to_clip=cam.world_to_clip,
                   world_to_eye_norm=cam.world_to_eye_norm, position=verts,
                   faces=np.arange(6, dtype=np.int32).reshape(2, 3))
    spec.normal = np.tile(np.array((0, 0, 1), F32), (6, 1))
    spec.colour = np.ones((6, 3), F32)
    spec.light_direction = np.array((0, 0, 1), F32)
    return spec


def test_ties_go_to_the_lowest_primitive():
    spec = _two_triangle_job(_lib.SHADER_GOURAUD)
    z0, c0 = scenes.initial_buffers(spec)
    out = oracle.render(spec, z0, c0)
    ids = out["prim_id"]
    assert (ids == 0).sum() > 10 and (ids == 1).sum() == 0
    assert out["near_ties"] == (ids == 0).sum()


def test_back_facing_first_primitive_fallback():
    # primitive 0 back-facing and alone: the default chooser falls back to
    # index 0; DepthShader (no front-facing test in its fragment) writes it,
    # Gouraud discards it (shader.py:215-217, gouraud.py:94-124).
    spec = _two_triangle_job(_lib.SHADER_DEPTH, second_offset=-50.0, flip_first=True)
    spec.faces = spec.faces[:1]
    z0, _ = scenes.initial_buffers(spec)
    out = oracle.render(spec, z0, None)
    assert (out["prim_id"] == 0).sum() > 10
    spec.shader = _lib.SHADER_GOURAUD
    z0, c0 = scenes.initial_buffers(spec)
    out = oracle.render(spec, z0, c0)
    assert (out["prim_id"] == 0).sum() == 0


@pytest.mark.parametrize("shader", scenes.ALL_SHADERS)
def test_every_shader_renders_something(shader):
    spec = scenes.random_job(shader, seed=shader)
    z0, c0 = scenes.initial_buffers(spec)
    out = oracle.render(spec, z0, c0)
    assert (out["prim_id"] >= 0).sum() > 0
    assert np.isfinite(out["zbuffer"]).all()


def test_double_twin_agrees_with_float():
    spec = scenes.random_job(_lib.SHADER_PHONG, seed=11)
    z0, c0 = scenes.initial_buffers(spec)
    a = oracle.render(spec, z0, c0)
    b = oracle.render(spec, z0, c0, dtype=np.float64)
    same = a["prim_id"] == b["prim_id"]
    assert same.mean() > 0.97
    np.testing.assert_allclose(a["canvas"][same], b["canvas"][same], atol=2e-3)


def test_column_band_equals_full_frame_columns():
    """The band-of-columns job the large-scene GPU test compares against
    (viewport x offset moved by -i0) renders exactly the full frame's columns."""
    from tests.test_gpu_workloads import band

    spec = scenes.random_job(_lib.SHADER_GOURAUD_TEXTURE, seed=5, W=64, H=40, F=200)
    z0, c0 = scenes.initial_buffers(spec)
    full = oracle.render(spec, z0, c0)
    for i0, w in ((0, 10), (20, 24), (50, 14)):
        b = oracle.render(band(spec, i0, w), z0[i0 : i0 + w], c0[i0 : i0 + w])
        np.testing.assert_array_equal(b["prim_id"], full["prim_id"][i0 : i0 + w])
        np.testing.assert_array_equal(b["zbuffer"].view(np.uint32), full["zbuffer"][i0 : i0 + w].view(np.uint32))
        np.testing.assert_array_equal(b["canvas"], full["canvas"][i0 : i0 + w])


def test_windowed_render_equals_the_full_render_inside_the_window():
    """The pixel window and the branch / texel probes used by the gradient
    checks (tests/fdgrad.py) change nothing inside the window."""
    from tests.scenes import random_job

    for shader in (_lib.SHADER_PHONG, _lib.SHADER_GOURAUD_TEXTURE, _lib.SHADER_PHONG_REFLECTION):
        spec = random_job(shader, seed=70 + shader, W=30, H=26, F=50)
        W, H = spec.width, spec.height
        full = oracle.render(spec, np.ones((W, H)), np.ones((W, H, 3)), dtype=np.float64, want_branch=True)
        plain = oracle.render(spec, np.ones((W, H)), np.ones((W, H, 3)), dtype=np.float64)
        assert np.array_equal(full["canvas"], plain["canvas"]) and np.array_equal(full["prim_id"], plain["prim_id"])
        win = (5, 17, 3, 20)
        part = oracle.render(spec, np.ones((W, H)), np.ones((W, H, 3)), dtype=np.float64, window=win, want_branch=True)
        sx, sy = slice(5, 17), slice(3, 20)
        for k in ("canvas", "zbuffer", "prim_id", "branch", "texel"):
            assert np.array_equal(part[k][sx, sy], full[k][sx, sy]), k
        outside = np.ones((W, H), bool)
        outside[sx, sy] = False
        assert (part["prim_id"][outside] == -1).all() and (part["canvas"][outside] == 1).all()
        kept = full["prim_id"] >= 0
        assert (full["texel"][kept] >= 0).all() and (full["texel"][~kept] == -1).all()
