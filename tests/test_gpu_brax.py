"""The notebooks' Brax pipeline on the GPU, on the reference's own Brax Ant
inputs (test_resources/pre-gen-brax/inputs-{2,30}.zip, committed as the
pickle-free archives tests/golden/brax_ant_{2,30}.npz by
tests/golden/make_brax_fixture.py): batched inputs -> instanced scenes ->
device merge -> tiled render through the fixtures' 960x540 camera (shadow
map of the canvas size through the camera viewport, centred on the
per-frame target) -> display epilogue; every frame at 84x84 (the notebooks'
benchmark size) and at the fixtures' own 960x540, against the oracle fed by
the host merge_objects path: winning primitives and depths bit-exact,
colours within 1e-5."""
import os
from pathlib import Path

import numpy as np
import pytest
import torch

from jaxrenderer_gb300 import _lib, batch as jb, brax
from jaxrenderer_gb300.utils import display_u8, transpose_for_display
from oracle import oracle
from tests.test_gpu_plain import assert_parity

pytestmark = pytest.mark.gpu
F32 = np.float32
GOLDEN = Path(__file__).resolve().parent / "golden"
THREADS = max(1, len(os.sched_getaffinity(0)))


def fixture(n_frames):
    return brax.load_batched_npz(GOLDEN / f"brax_ant_{n_frames}.npz")


def render(bb, W, H, device, tiled_config=None):
    sb, _ = brax.scene_batch(bb, W, H, device)
    out = jb.BatchRunner(sb, form="tiled", tiled_config=tiled_config).run()
    torch.cuda.synchronize()
    return out


def oracle_frame(bb, f, W, H):
    sub = bb.scenes.host_flat([f])
    shadow = bb.shadow._replace(centre=bb.shadow.centre[f : f + 1])
    tables = jb.scene_batch_tables(sub, W, H, bb.light, shadow, (W, H), bb.camera, shadow_viewport="camera")
    dspec, mspec = jb.scene_job_specs(sub, tables, 0)
    dref = oracle.render(dspec, np.full((W, H), np.finfo(F32).max, F32), n_threads=THREADS)
    mspec.shadow_map = dref["zbuffer"]
    ref = oracle.render(mspec, np.ones((W, H), F32), np.ones((W, H, 3), F32), n_threads=THREADS)
    return dref, ref


@pytest.mark.parametrize("n_frames,W,H", [(2, 84, 84), (30, 84, 84), (2, 960, 540), (30, 960, 540)])
def test_reference_brax_fixture_every_frame_matches_oracle(cuda_device, n_frames, W, H):
    objects, camera, target = fixture(n_frames)
    bb = brax.scenes_from_batched(objects, camera, target)
    assert bb.scenes.n_scenes == n_frames and bb.scenes.n_faces.tolist() == [3276] * n_frames
    out = render(bb, W, H, cuda_device)
    for f in range(n_frames):
        dref, ref = oracle_frame(bb, f, W, H)
        np.testing.assert_array_equal(out.shadow_map[f].cpu().numpy().view(np.uint32), dref["zbuffer"].view(np.uint32),
                                      err_msg=f"shadow map, frame {f}")
        assert_parity(out.zbuffer[f], out.canvas[f], out.prim_id[f], ref, f"frame {f} at {W}x{H}")
        assert (ref["prim_id"] >= 0).mean() > 0.2  # the scene is in view
        if W == 960:
            assert (ref["prim_id"] >= 12).sum() > 500  # capsule faces (ids past the ground's 12) are visible


def test_display_epilogue_on_the_reference_fixture(cuda_device):
    objects, camera, target = fixture(30)
    out = render(brax.scenes_from_batched(objects, camera, target, frames=[0, 7, 29]), 84, 84, cuda_device,
                 _lib.RastTiledConfig(8, 8, 0))
    got = display_u8(out.canvas).cpu().numpy()
    c = out.canvas.cpu().numpy()
    want = np.stack([transpose_for_display((np.clip(x, 0, 1) * 255).astype(np.uint8)) for x in c])
    np.testing.assert_array_equal(got, want)
    one = display_u8(out.canvas[1], flip_vertical=False).cpu().numpy()
    np.testing.assert_array_equal(one, transpose_for_display((np.clip(c[1], 0, 1) * 255).astype(np.uint8), False))

