"""Device-side merge_objects + per-corner flattening (rast_merge_objects)
against the host reference path (merge_objects + flatten_corners), bit for
bit, and instanced scenes rendered against the oracle."""
import numpy as np
import pytest
import torch

from jaxrenderer_gb300 import _lib, batch as jb, synthetic
from jaxrenderer_gb300.instancing import InstancedScenes, MeshLibrary
from jaxrenderer_gb300.model import Model
from oracle import oracle
from tests.test_gpu_plain import assert_parity

pytestmark = pytest.mark.gpu
F32 = np.float32


def stress_scenes(n_scenes=12, seed=0):
    """Meshes whose vertex, normal and uv counts differ, faces with
    out-of-range and negative indices (gathers wrap once, then clamp), an
    object without faces, and general (projective) transforms."""
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 60 + seed))
    box = synthetic.primitive_model("box", np.zeros(3, F32))
    ico = synthetic.primitive_model("icosphere2", np.zeros(3, F32))
    v = rng.normal(size=(9, 3)).astype(F32)
    n = rng.normal(size=(7, 3)).astype(F32)
    uv = rng.uniform(0, 4, (11, 2)).astype(F32)
    f = np.array([(0, 1, 2), (3, 4, 5), (6, 7, 8), (-1, 2, 12), (8, -3, 0)], np.int32)
    fn = np.array([(0, 1, 2), (3, 4, 5), (6, 0, 1), (-2, 9, 3), (1, 1, 1)], np.int32)
    fu = np.array([(0, 1, 2), (3, 4, 5), (6, 7, 8), (10, 13, -1), (9, 2, 40)], np.int32)
    odd = Model(v, n, uv, f, fn, fu, np.zeros((4, 4, 3), F32), np.full((4, 4), 2.0, F32))
    empty = Model(v[:3], n[:3], uv[:3], np.zeros((0, 3), np.int32), np.zeros((0, 3), np.int32),
                  np.zeros((0, 3), np.int32), np.zeros((4, 4, 3), F32), np.full((4, 4), 2.0, F32))
    lib = MeshLibrary.from_models([box, ico, odd, empty])
    counts = rng.integers(1, 7, n_scenes)
    I = int(counts.sum())
    mesh = rng.integers(0, 4, I).astype(np.int32)
    T = np.tile(np.identity(4, F32), (I, 1, 1))
    q = rng.normal(size=(I, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    T[:, :3, :3] = synthetic._quat_matrices(q)
    T[:, :3, 3] = rng.uniform(-2, 2, (I, 3))
    general = rng.random(I) < 0.3
    T[general] = rng.normal(size=(int(general.sum()), 4, 4)).astype(F32)
    T[general, 3, 3] += 3.0  # keep w away from 0 for most vertices
    scale = rng.uniform(0.3, 1.5, (I, 3)).astype(F32)
    diffuse = rng.uniform(0, 1, (I, 4, 4, 3)).astype(F32)
    specular = np.full((I, 4, 4), 2.0, F32)
    cam = np.tile(np.array([(4.0, 3.0, 2.0)], F32), (n_scenes, 1))
    return InstancedScenes(lib, mesh, np.concatenate([[0], np.cumsum(counts)]).astype(np.int64), T, scale,
                           diffuse, specular, cam)


def _bits(t):
    a = t.cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)
    return a.view(np.uint32) if a.dtype == np.float32 else a


def _check_pools(pools, flat):
    for name, host in (("position", flat.position), ("normal", flat.normal), ("uv", flat.uv),
                       ("texture_index", flat.texture_index)):
        np.testing.assert_array_equal(_bits(pools[name]), _bits(host), err_msg=name)


@pytest.mark.parametrize("which", ["brax", "stress"])
def test_device_merge_matches_host_path(cuda_device, which):
    inst = synthetic.brax_like_instances(48, seed=synthetic.BASE_SEED + 33) if which == "brax" else stress_scenes()
    sb, merge = jb.scene_batch_from_instances(inst, 32, 32, device=cuda_device)
    torch.cuda.synchronize()
    _check_pools(sb.pools, inst.host_flat(range(inst.n_scenes)))


def test_merge_follows_new_transforms(cuda_device):
    inst = stress_scenes(n_scenes=6, seed=1)
    sb, merge = jb.scene_batch_from_instances(inst, 32, 32, device=cuda_device)
    rng = np.random.default_rng(5)
    inst.transforms[:, :3, 3] += rng.uniform(-0.5, 0.5, (inst.n_instances, 3)).astype(F32)
    inst.local_scaling *= F32(1.25)
    merge.merge(torch.from_numpy(inst.transforms).pin_memory(), torch.from_numpy(inst.local_scaling).pin_memory())
    torch.cuda.synchronize()
    _check_pools(sb.pools, inst.host_flat(range(inst.n_scenes)))


def test_instanced_render_matches_oracle(cuda_device):
    inst = synthetic.brax_like_instances(16, seed=synthetic.BASE_SEED + 34)
    sb, _ = jb.scene_batch_from_instances(inst, 84, 84, shadow_size=(128, 128), device=cuda_device)
    out = jb.BatchRunner(sb, form="tiled", tiled_config=_lib.RastTiledConfig(8, 8, 0)).run()
    for s in (0, 7, 15):
        sub = inst.host_flat([s])
        tables = jb.scene_batch_tables(sub, 84, 84, shadow_size=(128, 128))
        dspec, mspec = jb.scene_job_specs(sub, tables, 0)
        dref = oracle.render(dspec, np.full((128, 128), np.finfo(F32).max, F32))
        np.testing.assert_array_equal(_bits(out.shadow_map[s]), _bits(dref["zbuffer"]))
        mspec.shadow_map = dref["zbuffer"]
        ref = oracle.render(mspec, np.ones((84, 84), F32), np.ones((84, 84, 3), F32))
        assert_parity(out.zbuffer[s], out.canvas[s], out.prim_id[s], ref, f"instanced scene {s}")


def test_instanced_pipeline_matches_direct_renders(cuda_device):
    # five frames of moving objects through the double-buffered pipeline
    # (merge of frame k + 1 overlapping the render of frame k), each equal
    # bit for bit to a direct merge + render of the same transforms
    inst = synthetic.brax_like_instances(8, seed=synthetic.BASE_SEED + 36)
    pipe = jb.InstancedPipeline(inst, 40, 36, shadow_size=(48, 48), device=cuda_device)
    sb, merge = jb.scene_batch_from_instances(inst, 40, 36, shadow_size=(48, 48), device=cuda_device)
    runner = jb.BatchRunner(sb, form="tiled", want_prim_id=False)
    rng = np.random.default_rng(9)
    frames, outs = [], []
    for k in range(5):
        tr = inst.transforms.copy()
        tr[:, :3, 3] += rng.uniform(-0.3, 0.3, (inst.n_instances, 3)).astype(F32)
        sc = (inst.local_scaling * rng.uniform(0.8, 1.2, (inst.n_instances, 1))).astype(F32)
        frames.append((torch.from_numpy(tr).pin_memory(), torch.from_numpy(sc).pin_memory()))
        outs.append(torch.empty((inst.n_scenes, 40, 36, 3), dtype=torch.float32, pin_memory=True))
    for (tr, sc), out in zip(frames, outs):
        pipe.frame(tr, sc, out=out)
    pipe.synchronize()
    for k, (tr, sc) in enumerate(frames):
        merge.merge(tr, sc)
        want = runner.run().canvas
        torch.cuda.synchronize()
        np.testing.assert_array_equal(_bits(outs[k]), _bits(want), err_msg=f"frame {k}")
    assert not np.array_equal(_bits(outs[0]), _bits(outs[1]))
