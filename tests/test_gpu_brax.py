"""The notebooks' Brax pipeline on the GPU: batched reference-format inputs
-> instanced scenes -> device merge -> tiled render at 84x84 through the
960x540 camera (shadow map of the canvas size through the camera viewport,
centred on the per-frame target) -> display epilogue; against the oracle
fed by the host merge_objects path."""
import numpy as np
import pytest
import torch

from jaxrenderer_gb300 import _lib, batch as jb, brax, synthetic
from jaxrenderer_gb300.utils import display_u8, transpose_for_display
from oracle import oracle
from tests.test_gpu_plain import assert_parity

pytestmark = pytest.mark.gpu
F32 = np.float32
W = H = 84


@pytest.fixture(scope="module")
def ant(cuda_device):
    objects, camera, target = synthetic.ant_like_batched(4)
    bb = brax.scenes_from_batched(objects, camera, target)
    sb, merge = brax.scene_batch(bb, W, H, cuda_device)
    out = jb.BatchRunner(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0)).run()
    torch.cuda.synchronize()
    return bb, sb, out


def test_brax_frames_match_oracle(ant):
    bb, sb, out = ant
    for f in (0, 3):
        sub = bb.scenes.host_flat([f])
        shadow = bb.shadow._replace(centre=bb.shadow.centre[f : f + 1])
        tables = jb.scene_batch_tables(sub, W, H, bb.light, shadow, (W, H), bb.camera, shadow_viewport="camera")
        dspec, mspec = jb.scene_job_specs(sub, tables, 0)
        dref = oracle.render(dspec, np.full((W, H), np.finfo(F32).max, F32))
        np.testing.assert_array_equal(out.shadow_map[f].cpu().numpy().view(np.uint32), dref["zbuffer"].view(np.uint32))
        mspec.shadow_map = dref["zbuffer"]
        ref = oracle.render(mspec, np.ones((W, H), F32), np.ones((W, H, 3), F32))
        assert_parity(out.zbuffer[f], out.canvas[f], out.prim_id[f], ref, f"frame {f}")
        assert (ref["prim_id"] >= 0).mean() > 0.2  # the scene is in view


def test_display_epilogue(ant):
    _, _, out = ant
    got = display_u8(out.canvas).cpu().numpy()
    c = out.canvas.cpu().numpy()
    want = np.stack([transpose_for_display((np.clip(x, 0, 1) * 255).astype(np.uint8)) for x in c])
    np.testing.assert_array_equal(got, want)
    one = display_u8(out.canvas[1], flip_vertical=False).cpu().numpy()
    np.testing.assert_array_equal(one, transpose_for_display((np.clip(c[1], 0, 1) * 255).astype(np.uint8), False))


def test_brax_full_view_frame_matches_oracle(cuda_device):
    """The whole 960x540 view (capsules in sight), one frame."""
    objects, camera, target = synthetic.ant_like_batched(2)
    bb = brax.scenes_from_batched(objects, camera, target, frames=[1])
    sb, _ = brax.scene_batch(bb, 960, 540, cuda_device)
    out = jb.BatchRunner(sb, form="tiled").run()
    sub = bb.scenes.host_flat([0])
    tables = jb.scene_batch_tables(sub, 960, 540, bb.light, bb.shadow, (960, 540), bb.camera, shadow_viewport="camera")
    dspec, mspec = jb.scene_job_specs(sub, tables, 0)
    dref = oracle.render(dspec, np.full((960, 540), np.finfo(F32).max, F32))
    mspec.shadow_map = dref["zbuffer"]
    ref = oracle.render(mspec, np.ones((960, 540), F32), np.ones((960, 540, 3), F32))
    assert_parity(out.zbuffer[0], out.canvas[0], out.prim_id[0], ref, "full view")
    ids = ref["prim_id"]
    assert (ids >= 12).sum() > 1000  # capsule faces (ids past the ground's 12) are visible
