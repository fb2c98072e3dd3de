"""Scene sharding: partition properties, and the rank-side logic with two
gloo ranks on CPU (no GPU, no data-path collective)."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from jaxrenderer_gb300.shard import partition, scene_costs


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_covers_and_balances(world):
    rng = np.random.Generator(np.random.PCG64(5))
    faces = rng.integers(300, 16000, size=4096)
    costs = scene_costs(faces, np.full(4096, 84), np.full(4096, 84), 128 * 128)
    parts = partition(costs, world)
    assert parts[0][0] == 0 and parts[-1][1] == 4096
    assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
    loads = [costs[b:e].sum() for b, e in parts]
    assert max(loads) <= costs.sum() / world + costs.max()


def test_partition_small_and_empty():
    assert partition([], 3) == [(0, 0)] * 3
    assert partition([5.0], 2) in ([(0, 0), (0, 1)], [(0, 1), (1, 1)])


def _rank(rank, world, port, faces, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = scene_costs(faces, np.full(len(faces), 84), np.full(len(faces), 84), 128 * 128)
    b, e = partition(costs, world)[rank]
    mine = torch.tensor([b, e, int(np.asarray(faces[b:e]).sum())], dtype=torch.int64)
    got = [torch.zeros(3, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(got, mine)  # host-side bookkeeping only
    dist.barrier()
    if rank == 0:
        out.put([g.tolist() for g in got])
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_shards():
    faces = np.random.Generator(np.random.PCG64(6)).integers(300, 16000, size=257)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, faces, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (b0, e0, f0), (b1, e1, f1) = res
    assert b0 == 0 and e0 == b1 and e1 == 257
    assert f0 + f1 == int(faces.sum())


def _bench_rank(rank, world, port, n, out):
    """bench.py's own rank set-up: each rank builds its shard.partition range
    of one world * n scene batch (build_brax84 without a device) and the
    ranks add their frames as run_ours does."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    wl = bench.build_brax84(n, rank, None, world)
    begin, end = wl.config["shard"]
    t = torch.tensor([float(wl.frames)])
    dist.all_reduce(t)
    mine = torch.tensor([begin, end, int(wl.instances.n_faces.sum()), int(t.item())], dtype=torch.int64)
    got = [torch.zeros(4, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(got, mine)
    if rank == 0:
        out.put([g.tolist() for g in got])
    dist.destroy_process_group()


def test_bench_ranks_render_contiguous_shards_of_one_batch():
    from jaxrenderer_gb300 import synthetic

    n, world = 48, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 30500 + os.getpid() % 1000
    procs = [ctx.Process(target=_bench_rank, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = q.get(timeout=180)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    (b0, e0, f0, t0), (b1, e1, f1, t1) = res
    assert b0 == 0 and e0 == b1 and e1 == n * world  # contiguous, covering the one batch
    assert t0 == t1 == n * world  # the frames every rank reports
    everything = synthetic.brax_like_instances(n * world, seed=synthetic.BASE_SEED + 1)
    assert f0 + f1 == int(everything.n_faces.sum())
