"""GPU parity of the tiled form: identical results to the plain form and the
oracle, for every tile shape, with bin overflow forced, and under CUDA-graph
replay."""
import numpy as np
import pytest
import torch

import jaxrenderer_gb300 as jr
from jaxrenderer_gb300 import _lib, batch as jb, synthetic
from jaxrenderer_gb300.jobs import pack, render_plain, render_tiled, unpack
from oracle import oracle
from tests import scenes
from tests.test_gpu_plain import assert_parity

pytestmark = pytest.mark.gpu
F32 = np.float32
SHAPES = [(8, 8), (16, 8), (16, 16), (32, 8), (8, 32), (8, 4), (4, 8)]
# tiles rasterised by two warps, each taking half of the rows
TWO_WARP_SHAPES = [(8, 8, 2), (8, 16, 2), (16, 16, 2)]


def _tiled_job(spec, z0, c0, device, tile=(8, 8), cap=0, ties=False, small=0):
    packed = pack([spec], [z0], [c0], device, count_ties=ties)
    wpt = tile[2] if len(tile) > 2 else 1
    stats = render_tiled(packed, tile=tile[:2], bin_capacity=cap, small_area=small, warps_per_tile=wpt)
    z, c, p = unpack(packed, [spec])[0]
    return z, c, p, packed.near_ties, stats


@pytest.mark.parametrize("shader", scenes.ALL_SHADERS)
def test_tiled_random_scene_parity(cuda_device, shader):
    spec = scenes.random_job(shader, seed=700 + shader, W=57, H=45, F=150, spread=2.0)
    z0, c0 = scenes.initial_buffers(spec)
    ref = oracle.render(spec, z0, c0)
    for tile in ((8, 8), (16, 16, 2)):
        z, c, p, ties, stats = _tiled_job(spec, z0, c0, cuda_device, tile=tile, ties=True)
        assert_parity(z, c, p, ref, f"tiled shader {shader} tile {tile}")
        assert int(ties.item()) == ref["near_ties"]
        assert stats.overflow == 0


@pytest.mark.parametrize("shader", scenes.ALL_SHADERS)
def test_small_face_path_parity(cuda_device, shader):
    # small faces rasterised by the setup kernel (atomicMin of packed keys)
    # and large ones binned, in one render: identical results
    spec = scenes.random_job(shader, seed=720 + shader, W=61, H=47, F=400, spread=2.5)
    z0, c0 = scenes.initial_buffers(spec)
    for tile in ((8, 8), (16, 16)):
        z, c, p, _, stats = _tiled_job(spec, z0, c0, cuda_device, tile=tile, small=32)
        assert_parity(z, c, p, oracle.render(spec, z0, c0), f"small path shader {shader} tile {tile}")


@pytest.mark.parametrize("tile", SHAPES + TWO_WARP_SHAPES)
def test_tile_shapes_and_unbounded_regions(cuda_device, tile):
    # eye inside the soup: many primitives straddle w = 0, so their coverage
    # regions are unbounded and must be clipped to the screen, not dropped
    spec = scenes.random_job(_lib.SHADER_PHONG, seed=800, W=70, H=50, F=300, spread=3.0, eye=(0.2, 0.1, 0.6))
    z0, c0 = scenes.initial_buffers(spec)
    z, c, p, _, _ = _tiled_job(spec, z0, c0, cuda_device, tile=tile)
    assert_parity(z, c, p, oracle.render(spec, z0, c0), f"tile {tile}")


def test_bin_overflow_falls_back_to_full_scan(cuda_device):
    spec = scenes.random_job(_lib.SHADER_GOURAUD, seed=801, W=64, H=64, F=400, spread=1.0)
    z0, c0 = scenes.initial_buffers(spec)
    z, c, p, _, stats = _tiled_job(spec, z0, c0, cuda_device, cap=64)
    assert stats.overflow == 1 and stats.bin_entries > 64
    assert_parity(z, c, p, oracle.render(spec, z0, c0), "overflow")


def test_reference_smoke_scene_tiled(cuda_device):
    spec = scenes.smoke_batched_triangles_job()
    z0 = np.ones((1920, 1080), F32)
    c0 = np.zeros((1920, 1080, 3), F32)
    z, c, p, _, _ = _tiled_job(spec, z0, c0, cuda_device, tile=(16, 16))
    scenes.smoke_batched_triangles_asserts(z.cpu().numpy(), c.cpu().numpy())
    assert_parity(z, c, p, oracle.render(spec, z0, c0, n_threads=8), "smoke tiled")


@pytest.fixture(scope="module")
def brax_batch(cuda_device):
    flat = synthetic.brax_like_batch(48, seed=synthetic.BASE_SEED + 21)
    sb = jb.scene_batch_from_flat(flat, 84, 84, shadow_size=(128, 128), device=cuda_device)
    return flat, sb


def _copy(out):
    keys = ("canvas", "zbuffer", "prim_id", "shadow_map", "shadow_prim_id")
    return {k: getattr(out, k).clone() for k in keys}


@pytest.mark.parametrize("tile,small", [((8, 8), 0), ((16, 16), 0), ((32, 8), 0), ((8, 4), 0), ((4, 8), 0),
                                        ((8, 8), 32), ((16, 8), 32), ((8, 4), 32),
                                        ((8, 16, 2), 0), ((16, 16, 2), 32), ((8, 8, 2), 0)])
def test_tiled_batch_equals_plain_batch(cuda_device, brax_batch, tile, small):
    flat, sb = brax_batch
    plain = _copy(jb.BatchRunner(sb, form="plain").run())
    cfg = _lib.RastTiledConfig(tile[0], tile[1], 0, small, tile[2] if len(tile) > 2 else 1)
    runner = jb.BatchRunner(sb, form="tiled", tiled_config=cfg)
    tiled = _copy(runner.run())
    torch.cuda.synchronize()
    for k in ("prim_id", "shadow_prim_id"):
        assert torch.equal(plain[k], tiled[k]), k
    for k in ("zbuffer", "shadow_map", "canvas"):
        assert torch.equal(plain[k].view(torch.int32), tiled[k].view(torch.int32)), k
    assert runner.stats("main").overflow == 0


def test_tiled_batch_matches_oracle_on_a_few_scenes(cuda_device, brax_batch):
    flat, sb = brax_batch
    out = jb.BatchRunner(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0)).run()
    torch.cuda.synchronize()
    for s in (0, 17, 47):
        dspec, mspec = scenes.specs_from_batch(flat, sb, s)
        dref = oracle.render(dspec, np.full((128, 128), np.finfo(F32).max, F32))
        np.testing.assert_array_equal(out.shadow_prim_id[s].cpu().numpy(), dref["prim_id"])
        mspec.shadow_map = dref["zbuffer"]
        ref = oracle.render(mspec, np.ones((84, 84), F32), np.ones((84, 84, 3), F32))
        assert_parity(out.zbuffer[s], out.canvas[s], out.prim_id[s], ref, f"scene {s}")


def test_graph_replay_matches_eager(cuda_device, brax_batch):
    flat, sb = brax_batch
    runner = jb.BatchRunner(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0))
    eager = _copy(runner.run())
    runner.capture()
    runner.canvas.zero_()
    replayed = runner.replay()
    torch.cuda.synchronize()
    assert torch.equal(eager["canvas"].view(torch.int32), replayed.canvas.view(torch.int32))
    assert torch.equal(eager["prim_id"], replayed.prim_id)


def adversarial_job(shader, seed, W=72, H=56):
    """Faces made to stress the conservative coverage rectangle: slivers
    (nearly parallel edges), sub-pixel triangles at pixel centres, corners
    exactly on pixel coordinates, huge triangles reaching far off screen,
    faces crossing w = 0 or with a corner at tiny w, needles across the
    frame, and repeated vertices.  world_to_clip maps (x, y, z) to
    (x, y, z, z) so each corner's w is its z."""
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + seed))
    vp = jr.Camera.viewport_matrix(np.zeros(2, np.int32), np.array((W, H)), 1.0).astype(F32)
    w2c = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 1, 0]], F32)
    # NDC of pixel (i, j) as the kernels compute it: x = (i - vp[0, 3]) / vp[0, 0]
    def ndc(i, j):
        return F32((F32(i) - vp[0, 3]) / vp[0, 0]), F32((F32(j) - vp[1, 3]) / vp[1, 1])

    tris = []
    for _ in range(60):  # slivers: a long edge and a third corner a hair off it
        p = rng.uniform(-1.2, 1.2, 2)
        d = rng.normal(size=2)
        d /= np.linalg.norm(d)
        n = np.array([-d[1], d[0]])
        L = rng.uniform(0.3, 2.5)
        eps = 10.0 ** rng.uniform(-7, -2)
        tris.append([p, p + L * d, p + rng.uniform(0.1, 0.9) * L * d + eps * n])
    for _ in range(60):  # sub-pixel triangles around pixel centres
        cx, cy = ndc(rng.integers(0, W), rng.integers(0, H))
        s = 10.0 ** rng.uniform(-5, -1.5)
        tris.append([np.array((cx, cy)) + s * rng.normal(size=2) for _ in range(3)])
    for _ in range(40):  # corners exactly on pixel coordinates
        tris.append([np.array(ndc(rng.integers(-2, W + 2), rng.integers(-2, H + 2))) for _ in range(3)])
    for _ in range(20):  # huge triangles
        tris.append([rng.uniform(-1e3, 1e3, 2) for _ in range(3)])
    for _ in range(20):  # needles across the frame
        a = rng.uniform(-1.5, 1.5, 2)
        b = -a + rng.normal(scale=0.01, size=2)
        tris.append([a, b, b + rng.normal(scale=1e-4, size=2)])
    for _ in range(10):  # a repeated corner (det 0: never kept)
        a, b = rng.uniform(-1, 1, 2), rng.uniform(-1, 1, 2)
        tris.append([a, a, b])
    verts, faces = [], []
    for k, t in enumerate(tris):
        z = rng.uniform(0.5, 3.0, 3)
        if k % 7 == 3:  # one corner behind the eye: the face crosses w = 0
            z[rng.integers(0, 3)] = -rng.uniform(0.05, 2.0)
        if k % 11 == 5:  # a corner at tiny positive w: huge projected coordinates
            z[rng.integers(0, 3)] = 10.0 ** rng.uniform(-6, -3)
        for q in range(3):
            verts.append((t[q][0] * z[q], t[q][1] * z[q], z[q]))  # NDC (x, y) at w = z
        faces.append((3 * k, 3 * k + 1, 3 * k + 2))
    verts = np.asarray(verts, F32)
    faces = np.asarray(faces, np.int32)
    rng.shuffle(faces)
    spec = jr.jobs.JobSpec(shader=shader, width=W, height=H, viewport=vp, world_to_clip=w2c,
                           world_to_eye_norm=np.identity(4, dtype=F32), position=verts, faces=faces)
    if shader == _lib.SHADER_GOURAUD:
        spec.normal = scenes.unit(rng, verts.shape[0])
        spec.colour = rng.uniform(0.0, 1.0, (verts.shape[0], 3)).astype(F32)
        spec.light_direction = np.array((0.3, 0.4, -0.8), F32)
    return spec


@pytest.mark.parametrize("shader", [_lib.SHADER_DEPTH, _lib.SHADER_GOURAUD])
def test_adversarial_faces_tiled_equals_plain_and_oracle(cuda_device, shader):
    spec = adversarial_job(shader, seed=900 + shader)
    z0, c0 = scenes.initial_buffers(spec)
    ref = oracle.render(spec, z0, c0)
    assert (ref["prim_id"] >= 0).sum() > 100
    packed = pack([spec], [z0], [c0], cuda_device, count_ties=True)
    render_plain(packed)
    zp, cp, pp = (None if t is None else t.clone() for t in unpack(packed, [spec])[0])
    assert_parity(zp, cp, pp, ref, f"plain adversarial shader {shader}")
    for tile in SHAPES + TWO_WARP_SHAPES:
        for small in (0, 32):
            z, c, p, _, stats = _tiled_job(spec, z0, c0, cuda_device, tile=tile, small=small)
            assert stats.overflow == 0
            assert torch.equal(p, pp), (tile, small)
            assert torch.equal(z.view(torch.int32), zp.view(torch.int32)), (tile, small)
            if c is not None:
                assert torch.equal(c.view(torch.int32), cp.view(torch.int32)), (tile, small)


def test_ragged_edge_case_batch(cuda_device):
    """One tiled batch of awkward jobs: no faces, a 1x1 and a 1-row canvas, a
    single face, reversed windings, an odd non-square canvas, a layered
    "over" job: every job equals the plain form and the oracle, for several
    tile shapes."""
    specs = []
    s = scenes.random_job(_lib.SHADER_GOURAUD, seed=950, W=20, H=20, F=30)
    s.faces = np.zeros((0, 3), np.int32)
    specs.append(s)
    specs.append(scenes.random_job(_lib.SHADER_PHONG, seed=951, W=1, H=1, F=40, spread=0.3))
    specs.append(scenes.random_job(_lib.SHADER_DEPTH, seed=952, W=37, H=1, F=40, spread=0.8))
    one = scenes.random_job(_lib.SHADER_GOURAUD_TEXTURE, seed=953, W=16, H=12, F=5, spread=0.8)
    one.faces = one.faces[:1]
    specs.append(one)
    flipped = scenes.random_job(_lib.SHADER_GOURAUD, seed=954, W=24, H=24, F=30, spread=0.8)
    flipped.faces = np.ascontiguousarray(flipped.faces[:, ::-1])  # every winding reversed
    specs.append(flipped)
    specs.append(scenes.random_job(_lib.SHADER_PHONG_REFLECTION, seed=955, W=7, H=93, F=80, spread=1.0))
    over = scenes.random_job(_lib.SHADER_PHONG_REFLECTION, seed=956, W=30, H=22, F=60, spread=0.9)
    over.layers, over.mixer, over.opacity = 3, _lib.MIX_OVER, 0.5
    specs.append(over)
    bufs = [scenes.initial_buffers(s) for s in specs]
    refs = [oracle.render(s, *b) for s, b in zip(specs, bufs)]
    assert (refs[0]["prim_id"] == -1).all() and (refs[5]["prim_id"] >= 0).any()
    for form, tile in (("plain", None), ("tiled", (8, 8)), ("tiled", (4, 8)), ("tiled", (16, 8)),
                       ("tiled", (16, 16, 2)), ("tiled", (8, 16, 2))):
        packed = pack(specs, [b[0] for b in bufs], [b[1] for b in bufs], cuda_device)
        if form == "plain":
            render_plain(packed)
        else:
            assert render_tiled(packed, tile=tile[:2], warps_per_tile=tile[2] if len(tile) > 2 else 1).overflow == 0
        for k, (s, out) in enumerate(zip(specs, unpack(packed, specs))):
            assert_parity(*out, refs[k], f"{form} {tile} job {k}")


def test_autotune_through_the_c_abi(cuda_device, brax_batch):
    """rast_autotune picks a configuration the tiled form has a kernel for,
    caches it per workload class (the second call renders nothing), and the
    picked configuration renders what the plain form renders."""
    import ctypes

    flat, sb = brax_batch
    runner = jb.BatchRunner(sb, form="plain")
    plain = _copy(runner.run())
    lib = _lib.load()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    cfg = _lib.RastTiledConfig()
    assert lib.rast_autotune(ctypes.byref(runner.main_batch), stream, ctypes.byref(cfg)) == 0
    shape = (cfg.tile_w, cfg.tile_h, cfg.warps_per_tile)
    assert shape[2] in (1, 2) and shape[:2] in [s[:2] for s in SHAPES + TWO_WARP_SHAPES]
    assert cfg.bin_capacity > 0 and cfg.small_area in (0, 32)
    again = _lib.RastTiledConfig()
    assert lib.rast_autotune(ctypes.byref(runner.main_batch), stream, ctypes.byref(again)) == 0
    assert bytes(again) == bytes(cfg)
    tiled = jb.BatchRunner(sb, form="tiled", tiled_config=cfg)
    got = _copy(tiled.run())
    torch.cuda.synchronize()
    assert torch.equal(got["prim_id"], plain["prim_id"])
    assert torch.equal(got["canvas"].view(torch.int32), plain["canvas"].view(torch.int32))


@pytest.mark.parametrize("flip", [(-1, 1), (1, -1), (-1, -1)])
def test_mirrored_viewports_tiled_equals_plain_and_oracle(cuda_device, flip):
    """Viewports with a negative x and/or y scale: the pixel <-> NDC maps
    run backwards, so the per-face pixel rectangles, the per-tile NDC tables
    and the pair path's entry rectangles all see decreasing coordinates."""
    specs = []
    for k, sh in enumerate((_lib.SHADER_GOURAUD, _lib.SHADER_DEPTH, _lib.SHADER_PHONG_REFLECTION)):
        s = scenes.random_job(sh, seed=980 + k, W=53, H=38, F=300, spread=1.4)
        vp = np.asarray(s.viewport, F32).reshape(4, 4).copy()
        vp[0, 0] *= flip[0]
        vp[1, 1] *= flip[1]
        s.viewport = vp
        specs.append(s)
    bufs = [scenes.initial_buffers(s) for s in specs]
    refs = [oracle.render(s, *b) for s, b in zip(specs, bufs)]
    assert all((r["prim_id"] >= 0).sum() > 200 for r in refs)
    for form, tile, small in (("plain", None, 0), ("tiled", (8, 8), 0), ("tiled", (16, 8), 0),
                              ("tiled", (16, 16, 2), 0), ("tiled", (4, 8), 32)):
        packed = pack(specs, [b[0] for b in bufs], [b[1] for b in bufs], cuda_device)
        if form == "plain":
            render_plain(packed)
        else:
            st = render_tiled(packed, tile=tile[:2], small_area=small, warps_per_tile=tile[2] if len(tile) > 2 else 1)
            assert st.overflow == 0
        for k, (s, out) in enumerate(zip(specs, unpack(packed, specs))):
            assert_parity(*out, refs[k], f"{form} {tile} flip {flip} job {k}")
