"""GPU parity on the benchmark workloads beyond the 84x84 batch: the
389,120-triangle overdraw scene (tiled == plain bit-exact on the full frame,
near ties counted alike; the oracle on bands of columns, near ties
included) and the mixed-resolution / mixed-shader batch at its configured
triangle counts (log-uniform 100 .. 100,000 per scene) rendered through one
MultiRunner graph (tiled == plain, the oracle on the smallest and the
largest scenes of every resolution class, the largest also with its bins
forced to overflow; backward of both forms)."""
import copy
import os

import numpy as np
import pytest
import torch

from jaxrenderer_gb300 import _lib, batch as jb, synthetic
from jaxrenderer_gb300.jobs import JobSpec, pack, render_plain, render_tiled, unpack
from oracle import oracle
from tests.test_gpu_plain import assert_parity

pytestmark = pytest.mark.gpu
F32 = np.float32
CLASSES = [(32, 32), (84, 84), (480, 270)]
THREADS = max(1, len(os.sched_getaffinity(0)))


@pytest.fixture(scope="module")
def overdraw(cuda_device):
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 3))
    d, est = synthetic.overdraw_scene(rng)
    spec = JobSpec(shader=_lib.SHADER_GOURAUD_TEXTURE, **d)
    assert spec.n_faces == 389_120 and est > 10
    z0 = np.ones((spec.width, spec.height), F32)
    c0 = np.ones((spec.width, spec.height, 3), F32)
    out = {}
    for form in ("plain", "tiled", "tiled_small"):
        packed = pack([spec], [z0], [c0], cuda_device, count_ties=form != "tiled_small")
        if form == "plain":
            render_plain(packed)
        else:
            stats = render_tiled(packed, tile=(8, 8), small_area=32 if form == "tiled_small" else 0)
            assert stats.overflow == 0
        z, c, p = unpack(packed, [spec])[0]
        ties = int(packed.near_ties.item()) if packed.near_ties is not None else None
        out[form] = (z.clone(), c.clone(), p.clone(), ties)
    return spec, z0, c0, out


def test_overdraw_scene_tiled_equals_plain(overdraw):
    spec, _, _, out = overdraw
    (zp, cp, pp, tp), (zt, ct, pt, tt) = out["plain"], out["tiled"]
    assert torch.equal(pp, pt)
    assert torch.equal(zp.view(torch.int32), zt.view(torch.int32))
    assert torch.equal(cp.view(torch.int32), ct.view(torch.int32))
    assert tp == tt
    assert (pp >= 0).float().mean() > 0.5  # the spheres cover most of the frame
    zs, cs, ps, _ = out["tiled_small"]  # small faces rasterised by the setup kernel
    assert torch.equal(pp, ps)
    assert torch.equal(zp.view(torch.int32), zs.view(torch.int32))
    assert torch.equal(cp.view(torch.int32), cs.view(torch.int32))


def band(spec: JobSpec, i0: int, w: int) -> JobSpec:
    """Columns [i0, i0 + w) of `spec` as a job of width w: the viewport's x
    offset moves by -i0 (exact in FP32 for these integers), so pixel i of the
    band computes what pixel i0 + i of the full frame does."""
    b = copy.copy(spec)
    b.width = w
    vp = np.array(spec.viewport, F32, copy=True)
    vp[0, 3] = F32(vp[0, 3] - F32(i0))
    assert float(vp[0, 3]) == float(spec.viewport[0, 3]) - i0
    b.viewport = vp
    return b


@pytest.mark.parametrize("i0,w", [(468, 24), (150, 16)])
def test_overdraw_scene_band_matches_oracle_near_ties_included(cuda_device, overdraw, i0, w):
    """Bands of columns (the middle of the frame, where the spheres pile up
    and duplicates tie exactly, and one off centre): the full frame's pixels
    bit-exact, and the band rendered alone counts the oracle's near ties
    (the tie rule: shader.py:207-251, argmin, first index)."""
    spec, z0, c0, out = overdraw
    z, c, p, _ = out["tiled"]
    bspec = band(spec, i0, w)
    ref = oracle.render(bspec, z0[i0 : i0 + w], c0[i0 : i0 + w], n_threads=THREADS)
    assert_parity(z[i0 : i0 + w], c[i0 : i0 + w], p[i0 : i0 + w], ref, "overdraw band")
    for form in ("plain", "tiled"):
        packed = pack([bspec], [z0[i0 : i0 + w]], [c0[i0 : i0 + w]], cuda_device, count_ties=True)
        if form == "plain":
            render_plain(packed)
        else:
            render_tiled(packed, tile=(8, 8))
        assert int(packed.near_ties.item()) == ref["near_ties"], form
    if i0 == 468:
        assert ref["near_ties"] > 0  # the band holds ties


@pytest.fixture(scope="module")
def mixed(cuda_device):
    n = 36
    flat = synthetic.cube_scene_batch(n, seed=synthetic.BASE_SEED + 17, f_min=100, f_max=100_000)
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 16))
    res = np.arange(n) % 3
    rng.shuffle(res)
    shadow = rng.random(n) < 0.5
    groups = jb.mixed_scene_batches(flat, res, CLASSES, shadow, device=cuda_device)
    assert len(groups) == 3
    return flat, res, shadow, groups


def _outputs(outs):
    return [{k: (None if getattr(o, k) is None else getattr(o, k).clone())
             for k in ("canvas", "zbuffer", "prim_id", "shadow_map", "shadow_prim_id")} for o in outs]


def test_mixed_batch_graph_tiled_equals_plain(mixed):
    _, _, _, groups = mixed
    sbs = [sb for _, sb in groups]
    tiled = jb.MultiRunner(sbs, form="tiled")
    tiled.capture()
    got = _outputs(tiled.replay())
    want = _outputs(jb.MultiRunner(sbs, form="plain").run())
    torch.cuda.synchronize()
    for g, w in zip(got, want):
        for k in g:
            if w[k] is None:
                assert g[k] is None
                continue
            a, b = g[k], w[k]
            if a.dtype == torch.float32:
                a, b = a.view(torch.int32), b.view(torch.int32)
            assert torch.equal(a, b), k


def test_mixed_batch_matches_oracle(mixed):
    flat, res, shadow, groups = mixed
    assert int(flat.n_faces.max()) >= 80_000 and int((flat.n_faces >= 50_000).sum()) >= 3
    for c, (idx, sb) in enumerate(groups):
        w, h = CLASSES[c]
        sub = synthetic.flat_subset(flat, idx)
        tables = jb.scene_batch_tables(sub, w, h, shadow_size=(w, h), shadow_mask=shadow[idx])
        out = jb.MultiRunner([sb], form="tiled").run()[0]
        # the cheapest scene with and the cheapest without a shadow pass, and the largest scene
        picks = []
        for want in (True, False):
            cand = [k for k in np.argsort(sub.n_faces) if bool(shadow[idx[k]]) == want]
            if cand:
                picks.append(int(cand[0]))
        picks.append(int(np.argmax(sub.n_faces)))
        for k in picks:
            dspec, mspec = jb.scene_job_specs(sub, tables, k)
            if dspec is not None:
                dref = oracle.render(dspec, np.full((w, h), np.finfo(F32).max, F32), n_threads=THREADS)
                srow = int(tables.shadow_index[k])
                np.testing.assert_array_equal(out.shadow_map[srow].cpu().numpy().view(np.uint32),
                                              dref["zbuffer"].view(np.uint32))
                mspec.shadow_map = dref["zbuffer"]
            ref = oracle.render(mspec, np.ones((w, h), F32), np.ones((w, h, 3), F32), n_threads=THREADS)
            assert_parity(out.zbuffer[k], out.canvas[k], out.prim_id[k], ref,
                          f"class {w}x{h} scene {k} ({int(sub.n_faces[k])} faces)")


def test_largest_mixed_scene_with_overflowing_bins_matches_oracle(cuda_device, mixed):
    """The largest 480x270 scene of the batch (tens of thousands of
    triangles) rendered with a bin capacity far below what it requests:
    tiles whose bins overflow fall back to a scan of the whole job, with the
    same results."""
    flat, res, shadow, groups = mixed
    c = 2
    idx, _ = groups[c]
    w, h = CLASSES[c]
    sub = synthetic.flat_subset(flat, idx)
    k = int(np.argmax(sub.n_faces))
    tables = jb.scene_batch_tables(sub, w, h, shadow_size=(w, h), shadow_mask=np.zeros(len(idx), bool))
    _, mspec = jb.scene_job_specs(sub, tables, k)
    z0, c0 = np.ones((w, h), F32), np.ones((w, h, 3), F32)
    packed = pack([mspec], [z0], [c0], cuda_device)
    full = render_tiled(packed, tile=(16, 16), bin_capacity=64 * mspec.n_faces)
    assert full.overflow == 0 and full.bin_entries > 10_000
    small = pack([mspec], [z0], [c0], cuda_device)
    st = render_tiled(small, tile=(16, 16), bin_capacity=int(full.bin_entries // 8))
    assert st.overflow == 1
    ref = oracle.render(mspec, z0, c0, n_threads=THREADS)
    for pk, what in ((packed, "fitting bins"), (small, "overflowing bins")):
        zz, cc, pp = unpack(pk, [mspec])[0]
        assert_parity(zz, cc, pp, ref, f"{int(sub.n_faces[k])}-face scene, {what}")


def test_mixed_batch_backward_tiled_matches_plain(mixed):
    _, _, _, groups = mixed
    sbs = [sb for _, sb in groups]
    grads = {}
    for form in ("tiled", "plain"):
        mr = jb.MultiRunner(sbs, form=form)
        outs = mr.run()
        gen = torch.Generator().manual_seed(3)
        gc = [torch.randn(o.canvas.shape, generator=gen).to(o.canvas.device) for o in outs]
        grads[form] = [{k: v.clone() for k, v in g.items()} for g in mr.backward(gc)]
    torch.cuda.synchronize()
    for gt, gp in zip(grads["tiled"], grads["plain"]):
        for k in gt:
            # Both forms hand the backward the same winners, so only the order
            # of the FP32 atomic sums differs.  Per-scene terms add ~1e5 pixel
            # contributions of either sign: run to run (same form) they move
            # by up to 4e-7 of the tensor's largest entry (1.2e-4 at 352 on
            # the 480x270 class), hence atol 1e-6 of that entry.
            atol = max(1e-5, 1e-6 * float(gp[k].abs().max()))
            torch.testing.assert_close(gt[k], gp[k], rtol=1e-4, atol=atol, msg=k)
        assert gt["position"].abs().sum() > 0
