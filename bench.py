"""Benchmark: frames/s of the rasterisation path, tiled-batched vs plain GPU.

Default workload (`--workload brax84`, the headline): the reference's
Brax-style 84x84 benchmark as a seeded synthetic stand-in: 4096 scenes, each a
ground plane plus 8-32 objects drawn from {box 12 tris, icosphere level 2 320
tris, capsule 16x8 512 tris}, uneven triangle counts (mean ~5.7k per scene),
PhongReflectionShadowTextureShader with a 128x128 light-space depth map.  One
step renders every scene once: the depth pass of all scenes, then the main
pass of all scenes.  One frame is one scene's final canvas.

Other workloads (one JSON line each, same keys):
  cube640     one 640x480 create_cube image, phong_reflection (fwd only)
  overdraw960 one 960x540 scene of 389,120 triangles, gouraud_texture,
              mean overdraw ~18 (fwd only)
  phong128    256 differentiable 128x128 phong scenes (icosphere level 4 with
              Gaussian displacement, 64x64 textures): fwd, and fwd+bwd of an
              MSE loss against images of the unperturbed meshes with
              gradients w.r.t. positions, texture, light and camera position
  mixed1024   1024 scenes at {32x32, 84x84, 480x270} with 100..100k cube
              triangles (log-uniform), half with a shadow pass, one CUDA graph
              over the three resolution classes, fwd and fwd+bwd

    python bench.py [--workload W] [--steps K] [--warmup W] [--form plain|tiled] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput; `e2e`
is the same work through the public batch API with the scene inputs copied
from pinned host memory and the canvases copied back inside the timed region.
`--impl reference` times the CPU oracle (the C restatement of the reference's
JAX path) on a bounded sample of the same workload, with all host threads.
"""
from __future__ import annotations

import argparse
import copy
import json
import os
import statistics
import subprocess
import sys
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Callable, Optional

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "frames/s @84x84x4096 scenes fwd and fwd+bwd, tiled-batched vs plain GPU"
UNIT = "frames/s"
L2_BYTES = 129 * 1024 * 1024
MIXED_CLASSES = [(32, 32), (84, 84), (480, 270)]
WORKLOADS = ("brax84", "ant84", "cube640", "overdraw960", "phong128", "mixed1024", "glass84")
DEFAULT_SCENES = {"brax84": 4096, "ant84": 200, "cube640": 1, "overdraw960": 1, "phong128": 256, "mixed1024": 1024,
                  "glass84": 4096}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=WORKLOADS, default="brax84")
    p.add_argument("--form", choices=["plain", "tiled", "auto"], default="auto")
    p.add_argument("--scenes", type=int, default=None)
    p.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of oracle work for cpu_baseline")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-bwd", action="store_true")
    p.add_argument("--tile-config", default=None,
                   help="pin the tiled form's config per pass instead of the autotuner's, e.g. "
                        "shadow=16x8,main=8x8x1 (width x height [x warps per tile]; bin capacity sized from a first render)")
    a = p.parse_args()
    if a.scenes is None:
        a.scenes = DEFAULT_SCENES[a.workload]
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# --------------------------------------------------------------- workloads

@dataclass
class Workload:
    key: str
    desc: str
    frames: int  # frames (scene canvases) per step
    chain: Callable[[int], tuple]  # scene k -> (depth JobSpec or None, main JobSpec), for the oracle
    work: np.ndarray  # per scene: pixel-triangle pairs of its passes (oracle cost model)
    groups: list = field(default_factory=list)  # SceneBatches on the device
    bwd: Optional[str] = "mse"  # fwd+bwd loss: "mse" against a fixed image, "phong", or None
    oracle_crop: int = 1  # the oracle renders width // oracle_crop columns of a frame
    config: dict = field(default_factory=dict)
    phong: Optional[dict] = None
    merges: list = field(default_factory=list)  # instancing.DeviceMerge per group (instanced workloads)
    instances: object = None  # instancing.InstancedScenes
    notebook: bool = False  # step = device merge + render + uint8 display epilogue, as the notebooks time it
    published: Optional[float] = None  # the reference's published frames/s for this configuration
    display: object = None  # uint8 display images of the notebook step
    api_inputs: object = None  # (objects, camera, target, light) host arrays for the get_camera_image e2e
    pinned: Optional[dict] = None  # {pass: RastTiledConfig} from --tile-config
    pipeline: Optional[Callable[[], object]] = None  # builds a batch.InstancedPipeline (instanced workloads)
    data: str = "synthetic (seeded stand-ins with the stated shapes)"


def _pass_work(spec) -> float:
    return float(spec.width) * spec.height * spec.n_faces if spec is not None else 0.0


def build_brax84(n, rank, dev, world=1):
    """The 4096-scene brax-like batch; with N ranks, one batch of N x 4096
    scenes split into N contiguous cost-balanced ranges (shard.partition),
    rank r rendering range r."""
    from jaxrenderer_gb300 import batch as jb, shard, synthetic

    W = H = 84
    shadow = (128, 128)
    everything = synthetic.brax_like_instances(n * world, seed=synthetic.BASE_SEED + 1)
    costs = shard.scene_costs(everything.n_faces, W, H, shadow[0] * shadow[1])
    begin, end = shard.partition(costs, world)[rank]
    inst = everything.subset(begin, end) if world > 1 else everything
    n = end - begin
    n_faces = inst.n_faces
    work = n_faces.astype(np.float64) * (W * H + shadow[0] * shadow[1])

    def chain(k):  # the host reference path for one scene: merge_objects + flatten_corners
        sub = inst.host_flat([k % n])
        return jb.scene_job_specs(sub, jb.scene_batch_tables(sub, W, H, shadow_size=shadow), 0)

    groups, merges = [], []
    if dev is not None:
        sb, merge = jb.scene_batch_from_instances(inst, W, H, shadow_size=shadow, device=dev)
        groups, merges = [sb], [merge]
    return Workload("brax84", "brax-like 84x84 x 4096 scenes, phong_reflection_shadow + 128x128 depth pass", n,
                    chain, work, groups, merges=merges, instances=inst,
                    config={"scenes": n, "mean_faces_per_scene": float(n_faces.mean()),
                            "objects": int(inst.n_instances), "resolution": [W, H], "shadow_map": list(shadow),
                            "shard": [int(begin), int(end)] if world > 1 else None},
                    pipeline=lambda prepare=None: jb.InstancedPipeline(inst, W, H, shadow_size=shadow, device=dev,
                                                                       prepare=prepare))


GLASS = {"layers": 4, "opacity": 0.6, "background": (0.55, 0.7, 0.9)}


def build_glass84(n, rank, dev, world=1):
    """The brax-like 84x84 batch through the compiled chooser / mix hooks:
    the 4 nearest candidates of every pixel blended front to back with
    opacity 0.6 over a sky colour (timed forward only)."""
    from jaxrenderer_gb300 import _lib, batch as jb

    wl = build_brax84(n, rank, dev, world)
    hooks = dict(layers=GLASS["layers"], mixer=_lib.MIX_OVER, opacity=GLASS["opacity"],
                 background=GLASS["background"])
    for sb in wl.groups:
        jb.set_layers(sb, **hooks)
    brax_chain = wl.chain

    def chain(k):
        depth, main = brax_chain(k)
        for name, v in hooks.items():
            setattr(main, name, v)
        return depth, main

    wl.key, wl.chain, wl.bwd = "glass84", chain, None
    brax_pipeline = wl.pipeline
    wl.pipeline = lambda prepare=None: brax_pipeline(prepare=lambda sb: jb.set_layers(sb, **hooks))
    wl.desc = ("brax-like 84x84 x 4096 scenes, phong_reflection_shadow + 128x128 depth pass, layered chooser "
               "(4 nearest candidates) + over mixer (opacity 0.6)")
    wl.config["hooks"] = {"primitive_chooser": "LayeredChooser(4)", "mix": "OverMixer(opacity=0.6)"}
    return wl


def build_cube640(n, rank, dev, world=1):
    import jaxrenderer_gb300 as jr
    from jaxrenderer_gb300 import _lib, batch as jb
    from jaxrenderer_gb300.jobs import job_from_extra

    W, H = 640, 480
    F32 = np.float32
    cube = jr.create_cube(np.ones(3, F32), np.ones(2, F32), np.zeros((2, 2, 3), F32) + np.array([0, 0, 1], F32),
                          np.ones((2, 2), F32) * 2.0)
    params = jr.CameraParameters(viewWidth=W, viewHeight=H, position=np.array([2.0, 4.0, 1.0], F32))
    cam = jr.Renderer.create_camera_from_parameters(params)
    extra, fi = jr.Renderer._extra(jr.merge_objects([jr.ModelObject(model=cube)]), jr.LightParameters(), cam)
    spec = job_from_extra(_lib.SHADER_PHONG_REFLECTION, cam, extra, W, H)
    spec.faces = fi
    groups = [jb.scene_batch_from_specs([spec] * n, dev)] if dev is not None else []
    return Workload("cube640", f"create_cube 640x480 x {n}, phong_reflection (Renderer.get_camera_image)", n,
                    lambda k: (None, spec), np.full(n, _pass_work(spec)), groups, bwd=None,
                    config={"scenes": n, "faces": 12, "resolution": [W, H]})


def build_overdraw960(n, rank, dev, world=1):
    from jaxrenderer_gb300 import _lib, batch as jb, synthetic
    from jaxrenderer_gb300.jobs import JobSpec

    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 3 + rank))
    d, overdraw = synthetic.overdraw_scene(rng)
    spec = JobSpec(shader=_lib.SHADER_GOURAUD_TEXTURE, **d)
    groups = [jb.scene_batch_from_specs([spec] * n, dev)] if dev is not None else []
    return Workload("overdraw960", f"960x540 x {n}, 64 level-4 + 3 level-5 icospheres (389,120 tris), "
                    "gouraud_texture, 512x512 texture", n, lambda k: (None, spec), np.full(n, _pass_work(spec)),
                    groups, bwd=None, oracle_crop=16,
                    config={"scenes": n, "faces": int(spec.n_faces), "resolution": [spec.width, spec.height],
                            "estimated_overdraw": round(overdraw, 2)})


def build_phong128(n, rank, dev, world=1):
    from jaxrenderer_gb300 import batch as jb, synthetic

    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 40 + rank))
    scenes = [synthetic.phong_scene(rng, level=4, texture_size=64, sigma=0.05, radius=4.0) for _ in range(n)]
    specs = [synthetic.phong_job_spec(sc) for sc in scenes]
    groups = [jb.scene_batch_from_specs(specs, dev)] if dev is not None else []
    phong = None
    if dev is not None:
        base = jb.scene_batch_from_specs([synthetic.phong_job_spec(sc, position=sc.base_position) for sc in scenes],
                                         dev)
        phong = {"scenes": scenes, "base": base}
    return Workload("phong128", f"{n} x 128x128 phong (icosphere L4 + displacement, 64x64 texture), "
                    "MSE vs unperturbed render, grads wrt positions/texture/light/camera", n,
                    lambda k: (None, specs[k % n]), np.array([_pass_work(s) for s in specs]), groups, bwd="phong",
                    config={"scenes": n, "faces": 5120, "resolution": [128, 128], "texture": [64, 64]},
                    phong=phong)


def build_mixed1024(n, rank, dev, world=1):
    from jaxrenderer_gb300 import batch as jb, synthetic

    flat = synthetic.cube_scene_batch(n, seed=synthetic.BASE_SEED + 5 + rank)
    rng = np.random.Generator(np.random.PCG64(synthetic.BASE_SEED + 6 + rank))
    res = rng.integers(0, len(MIXED_CLASSES), n)
    shadow = rng.random(n) < 0.5
    px = np.array([w * h for w, h in MIXED_CLASSES], np.float64)[res]
    work = flat.n_faces.astype(np.float64) * px * np.where(shadow, 2.0, 1.0)
    host = {}

    def chain(k):
        k = k % n
        c = int(res[k])
        if c not in host:
            idx = np.nonzero(res == c)[0]
            sub = synthetic.flat_subset(flat, idx)
            w, h = MIXED_CLASSES[c]
            host[c] = (sub, jb.scene_batch_tables(sub, w, h, shadow_size=(w, h), shadow_mask=shadow[idx]),
                       {int(s): i for i, s in enumerate(idx)})
        sub, tables, local = host[c]
        return jb.scene_job_specs(sub, tables, local[k])

    groups = []
    if dev is not None:
        groups = [sb for _, sb in jb.mixed_scene_batches(flat, res, MIXED_CLASSES, shadow, device=dev)]
    counts = {f"{w}x{h}": int((res == c).sum()) for c, (w, h) in enumerate(MIXED_CLASSES)}
    return Workload("mixed1024", f"{n} mixed scenes {{32x32, 84x84, 480x270}}, 100..100k cube tris log-uniform, "
                    "50% phong_reflection / 50% phong_reflection_shadow, one CUDA graph", n, chain, work, groups,
                    config={"scenes": n, "per_class": counts, "mean_faces_per_scene": float(flat.n_faces.mean()),
                            "shadow_scenes": int(shadow.sum()), "shadow_map": "canvas size (Renderer.render)"})


ANT_FIXTURE = ROOT / "tests" / "golden" / "brax_ant_30.npz"


def build_ant84(n, rank, dev, world=1):
    """The notebooks' benchmark (84x84/A100.ipynb cells 4-7) on the
    reference's own Brax Ant frames (test_resources/pre-gen-brax/
    inputs-30.zip, held as the pickle-free archive tests/golden/
    brax_ant_30.npz): 18 objects / 3,276 triangles per frame, the 30 frames
    cycled to the batch, rendered into 84x84 canvases through the pickled
    960x540 camera with the notebook's light and per-frame shadow centre,
    then clamped, scaled to uint8 and transposed for display."""
    from jaxrenderer_gb300 import batch as jb, brax

    W = H = 84
    objects, camera, target = brax.load_batched_npz(ANT_FIXTURE)
    frames = [(k + rank * n) % 30 for k in range(n)]
    # the batch as the notebook's prepare_data makes it (frames cycled), for the get_camera_image e2e
    idx = np.asarray(frames)
    cyc = lambda a: np.ascontiguousarray(np.asarray(a)[idx])  # noqa: E731
    api_objects = [o._replace(model=type(o.model)(*(cyc(x) for x in o.model)), local_scaling=cyc(o.local_scaling),
                              transform=cyc(o.transform), double_sided=cyc(o.double_sided)) for o in objects]
    api_camera = type(camera)(*(cyc(x) for x in camera))
    bb = brax.scenes_from_batched(objects, camera, target, frames=frames)
    inst = bb.scenes
    work = inst.n_faces.astype(np.float64) * (2 * W * H)

    def chain(k):
        k = k % n
        sub = inst.host_flat([k])
        shadow = bb.shadow._replace(centre=bb.shadow.centre[k : k + 1])
        t = jb.scene_batch_tables(sub, W, H, bb.light, shadow, (W, H), bb.camera, shadow_viewport="camera")
        return jb.scene_job_specs(sub, t, 0)

    groups, merges = [], []
    if dev is not None:
        sb, merge = brax.scene_batch(bb, W, H, dev)
        groups, merges = [sb], [merge]
    wl = Workload("ant84", f"Brax Ant 84x84 x {n} frames (the reference's inputs-30.zip frames cycled; 18 objects, "
                    "3,276 tris; 960x540 camera), phong_reflection_shadow, device merge + render + uint8 display "
                    "per step", n, chain, work,
                    groups, merges=merges, instances=inst, notebook=True, published=888.6 if n == 200 else None,
                    data="reference fixture (test_resources/pre-gen-brax/inputs-30.zip as tests/golden/"
                         "brax_ant_30.npz)",
                    config={"scenes": n, "faces_per_scene": 3276, "resolution": [W, H],
                            "camera_viewport": [960, 540], "shadow_map": [W, H],
                            "published": "888.6 frames/s, A100, batch 200 (notebooks/84x84/A100.ipynb:1308)"})
    wl.api_inputs = (api_objects, api_camera, cyc(target), bb.light)
    return wl


BUILDERS = {"ant84": build_ant84, "brax84": build_brax84, "cube640": build_cube640, "overdraw960": build_overdraw960,
            "phong128": build_phong128, "mixed1024": build_mixed1024, "glass84": build_glass84}


# ------------------------------------------------------------ CPU baseline

def oracle_frame(wl: Workload, k: int, threads: int) -> float:
    """Render scene k's passes with the oracle (main pass cropped to
    width // oracle_crop columns); returns the pixel-triangle pairs done."""
    from oracle import oracle

    depth, main = wl.chain(k)
    done = 0.0
    if wl.oracle_crop > 1:
        main = copy.copy(main)
        main.width = max(1, main.width // wl.oracle_crop)
    if depth is not None:
        f32max = np.finfo(np.float32).max
        smap = oracle.render(depth, np.full((depth.width, depth.height), f32max, np.float32),
                             n_threads=threads)["zbuffer"]
        main = copy.copy(main)
        main.shadow_map = smap
        done += _pass_work(depth)
    oracle.render(main, np.ones((main.width, main.height), np.float32),
                  np.ones((main.width, main.height, 3), np.float32), n_threads=threads)
    return done + _pass_work(main)


def time_oracle(wl: Workload, budget_s: float, threads: int, start: int = 0):
    """Consecutive scenes with the oracle until `budget_s` is spent.
    Returns (scenes, seconds, pixel-triangle pairs done)."""
    done, work = 0, 0.0
    t0 = time.perf_counter()
    while True:
        work += oracle_frame(wl, start + done, threads)
        done += 1
        el = time.perf_counter() - t0
        if el >= budget_s:
            return done, el, work


def oracle_rate(wl: Workload, budget_s: float, threads: int, start: int = 0):
    """Frames/s of the whole workload extrapolated from a timed sample:
    sample pixel-triangle pairs per second, applied to the workload's total
    (exact for equal scenes, cost-weighted for uneven ones)."""
    done, el, work = time_oracle(wl, budget_s, threads, start)
    rate = work / el
    fps = wl.frames / (float(wl.work.sum()) / rate)
    return fps, done, el


def cpu_baseline_line(wl: Workload, budget_s: float):
    threads = len(os.sched_getaffinity(0))
    fps, done, el = oracle_rate(wl, budget_s, threads)
    crop = f", main pass cropped to 1/{wl.oracle_crop} of the columns" if wl.oracle_crop > 1 else ""
    return {"value": fps, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{done} consecutive scenes of the workload{crop}, oracle C restatement, OpenMP over pixel "
                      f"columns, {el:.1f} s; frames/s = sample pixel-triangle rate applied to the whole workload"}


# ------------------------------------------------------------------ clocks

class ClockSampler:
    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = ROOT / "gpurun_out" / f"clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ------------------------------------------------------------------- ours

INPUT_POOLS = ("position", "normal", "uv", "colour", "texture_index", "texture", "specular_map")


def input_bytes(groups) -> int:
    return sum(sb.pools[k].numel() * sb.pools[k].element_size() for sb in groups for k in INPUT_POOLS
               if k in sb.pools)


class Timer:
    """Device time of repeated steps: CUDA events on the launching stream,
    a barrier + synchronize on both sides, max over ranks.  With `flush`
    (inputs smaller than L2), a buffer larger than L2 is written before each
    step, outside the events."""

    def __init__(self, dev, stream, world, flush: bool):
        import torch

        self.torch = torch
        self.dev, self.stream, self.world = dev, stream, world
        self.scratch = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev) if flush else None

    def barrier(self):
        self.torch.cuda.synchronize(self.dev)
        if self.world > 1:
            self.torch.distributed.barrier()

    def __call__(self, step_fn, steps, warmup):
        torch = self.torch
        for _ in range(warmup):
            step_fn()
        self.barrier()
        ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
        if self.scratch is None:
            start, stop = ev(), ev()
            start.record(self.stream)
            for _ in range(steps):
                step_fn()
            stop.record(self.stream)
            self.barrier()
            ms = start.elapsed_time(stop)
        else:
            pairs = []
            for k in range(steps):
                self.scratch.fill_(float(k))
                a, b = ev(), ev()
                a.record(self.stream)
                step_fn()
                b.record(self.stream)
                pairs.append((a, b))
            self.barrier()
            ms = sum(a.elapsed_time(b) for a, b in pairs)
        if self.world > 1:
            t = torch.tensor([ms], device=self.dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms / steps


def run_ours(args, rank, world, local):
    import torch

    from jaxrenderer_gb300 import _lib, batch as jb

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    _lib.load()
    wl = BUILDERS[args.workload](args.scenes, rank, dev, world)
    stream = torch.cuda.current_stream(dev)
    form, form_times = args.form, None
    if args.form == "auto" and not args.tile_config:
        form, form_times = choose_form(wl, dev)
    elif args.form == "auto":
        form = "tiled"
    in_bytes = input_bytes(wl.groups)
    flush = in_bytes < 2 * L2_BYTES
    timed = Timer(dev, stream, world, flush)

    pinned = wl.pinned = pinned_configs(args.tile_config, wl.groups)
    mr = jb.MultiRunner(wl.groups, form=form, want_prim_id=False, tiled_config=pinned)
    if wl.notebook:
        step, wl.display = notebook_step(wl, mr, dev, capture=True)
    else:
        mr.capture()
        step = mr.replay
    with ClockSampler(local) as clk:  # sampled over the warm-up and the timed steps
        time.sleep(0.2)
        for _ in range(args.warmup):
            step()
        ms_per_step = timed(step, args.steps, 0)
    total_frames = wl.frames
    if world > 1:  # every rank's frames (equal under weak scaling, cost-balanced ranges for brax84)
        t = torch.tensor([float(wl.frames)], device=dev)
        torch.distributed.all_reduce(t)
        total_frames = int(t.item())
    value = total_frames / (ms_per_step / 1e3)
    prof = profile_kernels(mr, args.steps, stream)
    visible = count_visible(mr)

    comparison = {}
    if not args.no_plain:  # the plain form as the reference's method runs: eager, one pass per call
        plain = jb.MultiRunner(wl.groups, form="plain", want_prim_id=False)
        pms = timed(lambda: plain.run(stream), max(1, min(args.steps, 3)), 1)
        comparison = {"plain_fwd": total_frames / (pms / 1e3), "plain_ms_per_step": pms}
        if form == "tiled":
            comparison["tiled_over_plain"] = pms / ms_per_step
        else:  # small workload: the graph-replayed plain form was the faster
            comparison["tiled_graph_ms_per_step"] = form_times["tiled"]
            comparison["tiled_fwd"] = total_frames / (form_times["tiled"] / 1e3)
        del plain
        torch.cuda.empty_cache()

    fwd_bwd = {}
    if not args.no_bwd and wl.bwd is not None:
        fwd_bwd = measure_fwd_bwd(wl, args, stream, timed, total_frames)

    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(wl, mr, step, args, dev, stream, total_frames)
        if wl.notebook and world == 1:
            # the same frames through the reference's call, Renderer.get_camera_image on batched inputs
            api = measure_e2e_api(wl, args, dev, stream, total_frames)
            e2e = dict(api, pipelined=e2e)

    ties = count_near_ties(mr)
    kernels_per_step = prof["launches_per_step"]
    clocks = clk.summary()
    roof, per_kernel = roofline(prof, visible, clocks)
    detail = {"kernels": prof["summary"], "per_kernel": per_kernel,
              "backward_kernels_ms": fwd_bwd.pop("backward_kernels_ms", None), "fwd_bwd_grads": fwd_bwd.pop("grads", None)}
    detail_path = ROOT / "gpurun_out" / f"bench_{args.workload}_s{args.scenes}_n{world}_detail.json"
    if rank == 0:
        detail_path.parent.mkdir(exist_ok=True)
        detail_path.write_text(json.dumps(detail, indent=1))
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": (value / wl.published) if wl.published else None,
        "dtype": "f32",
        "data": wl.data,
        "config": dict({
            "workload": wl.desc,
            "form": form + " (CUDA graph replay)" + (
                "" if form_times is None else
                ", the faster of the two forms on this workload (" +
                ", ".join(f"{k} {v:.3f} ms" for k, v in form_times.items()) + " per step)"),
            "tiled_config": {name: [c.tile_w, c.tile_h, int(c.bin_capacity), int(c.small_area), int(c.warps_per_tile)]
                             for name, r, p in prof["passes"]
                             for c in [r.configs.get(p)] if c is not None},
            "l2": ("inputs larger than L2 (input pools %.2f GB)" % (in_bytes / 1e9)) if not flush else
                  ("L2 flushed between timed steps (a %d MB buffer written; input pools %.1f MB)"
                   % (2 * L2_BYTES >> 20, in_bytes / 1e6)),
            "parallelism": f"scene-sharded x{world} (no collective)",
        }, **wl.config),
        "fwd_tiled_over_plain": comparison.get("tiled_over_plain"),
        "fwd_bwd_tiled_over_plain": fwd_bwd.get("tiled_over_plain"),
        "fwd_bwd_value": fwd_bwd.get("tiled", {}).get("value"),
        "fwd_comparison": comparison,
        "fwd_bwd": fwd_bwd,
        "near_ties": ties,
        "roofline": roof,
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": clocks,
        "detail_file": str(detail_path.relative_to(ROOT)),
    }
    if e2e is not None:
        out["e2e"] = e2e
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_line(wl, budget_s=args.cpu_budget)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def count_near_ties(mr):
    """Pixels whose two best candidate depths lie within 1 ulp of each other
    (counted by the kernels, resolved exactly by the lowest primitive id), per
    pass, from one counting render of every scene in the timed form (the
    tiled form counts with its small-face path off)."""
    import torch

    from jaxrenderer_gb300 import batch as jb

    out = {"main": 0, "shadow": 0, "main_pixels": 0, "shadow_pixels": 0}
    for r in mr.runners:
        rr = jb.BatchRunner(r.sb, form=r.form, want_prim_id=False, count_ties=True, tiled_config=dict(r.configs) or None)
        rr.ties.zero_()
        rr.shadow_ties.zero_()
        rr.run()
        torch.cuda.synchronize()
        out["main"] += int(rr.ties.item())
        out["main_pixels"] += int(rr.canvas.shape[0] * rr.canvas.shape[1] * rr.canvas.shape[2])
        if rr.shadow_map is not None:
            out["shadow"] += int(rr.shadow_ties.item())
            out["shadow_pixels"] += int(rr.shadow_map.numel())
        del rr
    torch.cuda.empty_cache()
    return out


def measure_e2e_api(wl: Workload, args, dev, stream, total_frames):
    """The notebooks' step through the reference's own call: host-resident
    batched ModelObjects / CameraParameters / shadow centres ->
    Renderer.get_camera_image (one batch, set-up cached between calls, the
    transforms and job tables copied to the device every call) -> uint8
    display epilogue -> pinned host memory, all inside the timed region."""
    import torch

    import jaxrenderer_gb300 as jr
    from jaxrenderer_gb300.utils import display_u8

    objects, camera, target, light = wl.api_inputs
    W, H = wl.config["resolution"]
    shadow = jr.ShadowParameters(centre=target)
    n = int(np.asarray(target).shape[0])
    out_host = torch.empty((n, H, W, 3), dtype=torch.uint8, pin_memory=True)

    def api_step():
        img = jr.Renderer.get_camera_image(objects, light, camera, W, H, shadow_param=shadow)
        out_host.copy_(display_u8(img), non_blocking=True)

    api_step()  # first call: builds and caches the instanced set-up
    torch.cuda.synchronize(dev)
    steps = max(1, min(args.steps, 10))
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    start.record(stream)
    for _ in range(steps):
        api_step()
    stop.record(stream)
    torch.cuda.synchronize(dev)
    wall = (time.perf_counter() - t0) * 1e3 / steps
    ms = max(start.elapsed_time(stop) / steps, wall)
    n_obj = len(objects)
    h2d = n * n_obj * (16 + 3) * 4 + 2 * n * int(np.dtype(wl.groups[0].main_jobs.dtype).itemsize)
    return {"value": total_frames / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(out_host.numel()),
            "inputs": "Renderer.get_camera_image(batched ModelObjects, LightParameters, batched CameraParameters, "
                      "84, 84, shadow_param=ShadowParameters(centre=batched target)) on host arrays, the "
                      "notebooks' vmapped call: transforms, local scalings and job tables copied every call",
            "outputs": "uint8 display images (clamp, x255, transpose_for_display) to pinned host memory"}


def pinned_configs(spec: Optional[str], groups):
    """{pass: RastTiledConfig} from --tile-config ("shadow=16x8,main=8x8x1"),
    each with a bin capacity of 1.25x the entries a first render of the
    largest group requests; None without the option."""
    if not spec:
        return None
    import ctypes

    import torch

    from jaxrenderer_gb300 import _lib, batch as jb

    out = {}
    for item in spec.split(","):
        name, shape = item.split("=")
        dims = [int(v) for v in shape.lower().split("x")]
        out[name.strip()] = _lib.RastTiledConfig(dims[0], dims[1], 0, 0, dims[2] if len(dims) > 2 else 1)
    probe = jb.BatchRunner(max(groups, key=lambda sb: sb.n_scenes), form="tiled", want_prim_id=False,
                           tiled_config={k: _lib.RastTiledConfig.from_buffer_copy(v) for k, v in out.items()})
    for name, cfg in out.items():
        if name not in probe.configs:
            continue
        c = probe.configs[name]
        c.bin_capacity = 64 * int(probe.sb.total_faces)  # ample for the probe render
        nbytes = int(probe._ws_bytes(name, probe.shadow_batch if name == "shadow" else probe.main_batch))
        probe.ws[name] = (torch.empty(max(nbytes, 256), dtype=torch.uint8, device=probe.sb.device), nbytes)
    probe.run()
    for name, cfg in out.items():
        if name in probe.configs:
            cfg.bin_capacity = int(probe.stats(name).bin_entries * 1.25) + 4096
    del probe
    torch.cuda.empty_cache()
    return out


def choose_form(wl: Workload, dev):
    """The form `value` is timed with: tiled for large workloads; for small
    ones (under 1e9 pixel-triangle pairs, where the tiled form's fixed
    launch costs can dominate) the faster of both forms' graph replays.
    Both give identical results.  Returns (form, {form: ms per replay} or
    None)."""
    import torch

    from jaxrenderer_gb300 import batch as jb

    if wl.notebook or float(wl.work.sum()) >= 1e9:
        return "tiled", None
    times = {}
    for f in ("tiled", "plain"):
        mr = jb.MultiRunner(wl.groups, form=f, want_prim_id=False)
        mr.capture()
        for _ in range(3):
            mr.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            mr.replay()
        e1.record()
        torch.cuda.synchronize(dev)
        times[f] = e0.elapsed_time(e1) / 10
        del mr
    return min(times, key=times.get), times


def notebook_step(wl: Workload, mr, dev, capture: bool):
    """One step as the notebooks time it: rebuild the per-corner pools from
    the resident transforms (rast_merge_objects), render, and the uint8
    display epilogue (rast_display_u8); as one CUDA graph when `capture`."""
    import torch

    from jaxrenderer_gb300.utils import display_u8

    r = mr.runners[0]
    n, w, h, c = r.canvas.shape
    display = torch.empty((n, h, w, c), dtype=torch.uint8, device=dev)

    def step(stream=None):
        s = stream if stream is not None else torch.cuda.current_stream(dev)
        wl.merges[0].merge(stream=s)
        mr.run(s)
        display_u8(r.canvas, out=display, stream=s)

    if not capture:
        return step, display
    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    step(side)
    torch.cuda.current_stream(dev).wait_stream(side)
    torch.cuda.synchronize(dev)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()
    return g.replay, display


def count_visible(mr):
    """Faces that win at least one pixel of a main pass (the faces whose
    varyings the tiled form computes), per runner, from one prim-id render."""
    import torch

    from jaxrenderer_gb300 import batch as jb

    out = []
    for r in mr.runners:
        rr = jb.BatchRunner(r.sb, form=r.form, want_prim_id=True, tiled_config=dict(r.configs) or None)
        rr.run()
        pid = rr.prim_id.reshape(r.sb.n_scenes, -1).to(torch.int64)
        key = torch.arange(r.sb.n_scenes, device=pid.device)[:, None] * (1 << 32) + pid
        out.append(int(torch.unique(key[pid >= 0]).numel()))
        del rr, pid, key
    torch.cuda.empty_cache()
    return out


def measure_fwd_bwd(wl: Workload, args, stream, timed, total_frames):
    """Forward + backward per step.  "mse": MSE against a fixed image per
    scene: render (prim-id buffer saved), then rast_backward_mse into reused
    gradient arrays (per-vertex, per-texel, per-scene camera/light), zeroed
    first; it forms dL/dcanvas = (canvas - target) * 2/n per pixel inside the
    backward (no gradient image is written or read).
    "phong": the differentiable phong batch through DifferentiableBatch and
    torch autograd: camera matrices from eye positions, render, MSE against
    the unperturbed meshes' images, backward to positions, texture, light
    direction and camera position."""
    import torch

    from jaxrenderer_gb300 import _lib, batch as jb

    out = {}
    for form in ("tiled", "plain"):
        if form == "plain" and args.no_plain:
            continue
        steps = args.steps if form == "tiled" else max(1, min(args.steps, 3))
        warm = args.warmup if form == "tiled" else 1
        if wl.bwd == "phong":
            step, r, extra = phong_step(wl, form)
            runners = [r]
        else:
            mr = jb.MultiRunner(wl.groups, form=form, want_prim_id=True,
                                tiled_config=wl.pinned if form == "tiled" else None)
            grads = mr.grad_buffers()
            gen = torch.Generator().manual_seed(0)
            targets = [torch.rand(r.canvas.shape, generator=gen).to(r.canvas.device) for r in mr.runners]
            scales = [2.0 / t.numel() for t in targets]
            if form == "tiled":
                mr.capture()
                fwd = mr.replay
            else:
                fwd = lambda mr=mr: mr.run(stream)  # noqa: E731

            def step(mr=mr, fwd=fwd, grads=grads):
                fwd()
                mr.backward_mse(targets, scales, out=grads)

            runners = mr.runners
            mr = None
        ms = timed(step, steps, warm)
        out[form] = {"value": total_frames / (ms / 1e3), "ms_per_step": ms, "steps": steps}
        if form == "tiled":
            # backward alone, and its kernels (CUDA events inside the library)
            step()
            torch.cuda.synchronize()
            gcs = [(r.canvas - r.canvas.detach().mean()) * 1e-3 for r in runners]
            gbs = [r.grad_buffers() for r in runners]

            def bwd():
                for r, g, b in zip(runners, gcs, gbs):
                    r.backward(g, out=b)

            out["backward_ms"] = timed(bwd, steps, 1)
            kms = {}
            for r, g, b in zip(runners, gcs, gbs):
                prof = _lib.RastProfile()
                r.backward(g, out=b, profile=prof)
                for k in range(prof.n):
                    name = prof.names[k].decode()
                    kms[name] = kms.get(name, 0.0) + prof.ms[k]
            out["backward_kernels_ms"] = kms
            if wl.bwd == "phong":
                out["grads"] = extra()
        del step, runners
        torch.cuda.empty_cache()
    if "plain" in out:
        out["tiled_over_plain"] = out["plain"]["ms_per_step"] / out["tiled"]["ms_per_step"]
    out["unit"] = UNIT
    return out


def phong_step(wl: Workload, form: str):
    """One fwd+bwd step of the differentiable phong batch (see measure_fwd_bwd)."""
    import torch

    from jaxrenderer_gb300 import batch as jb, synthetic
    from jaxrenderer_gb300.autograd import DifferentiableBatch, camera_matrices

    sb = wl.groups[0]
    dev = sb.device
    scenes = wl.phong["scenes"]
    tr = jb.BatchRunner(wl.phong["base"], form=form, want_prim_id=False)
    target = tr.run().canvas.clone()
    del tr
    db = DifferentiableBatch(sb, form=form)
    params = synthetic.phong_camera_params(scenes[0].eye)
    eye = torch.tensor(np.stack([sc.eye for sc in scenes]), dtype=torch.float32, device=dev, requires_grad=True)
    light = torch.tensor(np.stack([sc.light_direction for sc in scenes]), dtype=torch.float32, device=dev,
                         requires_grad=True)
    pos = sb.pools["position"].clone().requires_grad_(True)
    tex = sb.pools["texture"].clone().requires_grad_(True)
    leaves = (eye, light, pos, tex)
    look_at = torch.zeros(3, dtype=torch.float32, device=dev)
    up = torch.tensor(np.asarray(params.up, np.float32), device=dev)

    def step():
        for t in leaves:
            t.grad = None
        w2c, w2e, _ = camera_matrices(eye, params, target=look_at, up=up)
        canvas, _ = db.render(position=pos, texture=tex, world_to_clip=w2c, world_to_eye_norm=w2e,
                              light_direction=light)
        loss = ((canvas - target) ** 2).mean()
        loss.backward()

    # the whole step (camera matrices, render, loss, backward) as one CUDA graph
    side = torch.cuda.Stream(dev)
    side.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(side):
        for _ in range(3):
            step()
    torch.cuda.current_stream(dev).wait_stream(side)
    torch.cuda.synchronize(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()

    def extra():
        return {k: float(t.grad.abs().sum()) if t.grad is not None else None
                for k, t in zip(("camera_position", "light_direction", "position", "texture"), leaves)}

    return graph.replay, db.runner, extra


def profile_kernels(mr, steps, stream):
    """Per-kernel CUDA-event durations inside the library, same steps again.
    Kernel names are "pass:kernel", prefixed by "WxH/" for multi-class runs."""
    from jaxrenderer_gb300 import _lib

    acc, names_order, passes, where = {}, [], [], {}
    multi = len(mr.runners) > 1
    launches = 0
    for it in range(steps):
        for r in mr.runners:
            r._reset(1.0)
            prefix = f"{r.sb.width}x{r.sb.height}/" if multi else ""
            for key, _b in r.batches():
                if it == 0:
                    passes.append((prefix + key, r, key))
                prof = _lib.RastProfile()
                r.launch(key, stream.cuda_stream, profile=prof)
                for k in range(prof.n):
                    kname = prof.names[k].decode()
                    name = f"{prefix}{key}:{kname}"
                    if name not in acc:
                        acc[name] = []
                        names_order.append(name)
                        where[name] = (r, key, kname)
                    acc[name].append(prof.ms[k])
                    if it == 0 and kname != "memset":
                        launches += 2 if kname == "scan_kernels" else 1
    summary = {n: {"avg_ms": float(np.mean(v)), "launches": len(v)} for n, v in acc.items()}
    total = sum(v["avg_ms"] for v in summary.values())
    for v in summary.values():
        v["share"] = v["avg_ms"] / total if total > 0 else 0.0
    return {"summary": summary, "order": names_order, "where": where, "passes": passes,
            "launches_per_step": launches}


# bytes a face corner's vertex inputs take, and texel bytes a pixel reads, per shader id
_CORNER_IN = {0: 12, 1: 36, 2: 32, 3: 32, 4: 32, 5: 36, 6: 36}
_TEXEL = {0: 0, 1: 0, 2: 12, 3: 12, 4: 24, 5: 16, 6: 20}
_VARYINGS = {0: 0, 1: 3, 2: 5, 3: 5, 4: 20, 5: 6, 6: 10}  # floats per corner (rast_shaders.cuh varying_count)


def pass_info(runner, pass_name):
    jobs = runner.sb.shadow_jobs if pass_name == "shadow" else runner.sb.main_jobs
    sh = jobs["shader"].astype(np.int64)
    px = jobs["width"].astype(np.int64) * jobs["height"]
    nv = jobs["n_verts"].astype(np.int64)
    info = {
        "F": float(jobs["n_faces"].astype(np.int64).sum()),
        "P": float(px.sum()),
        "Ptex": float(sum(px[k] * _TEXEL[int(sh[k])] for k in range(len(sh)))),
        "corners": float(nv.sum()),
        "cin": float(sum(nv[k] * _CORNER_IN[int(sh[k])] for k in range(len(sh)))),
        "vs": max(_VARYINGS[int(s)] for s in np.unique(sh)),
        "tests": float((px * jobs["n_faces"].astype(np.int64)).sum()),
        "main": bool((sh != 0).any()),
        "slots": 4 if int(jobs["layers"].max()) > 0 else 1,  # chooser slots written per pixel
        "E": 0.0,
        "T": 0.0,
        "B": 0.0,
    }
    if runner.form == "tiled":
        st = runner.stats(pass_name)
        info["E"], info["T"], info["B"] = float(st.bin_entries), float(st.tiles), float(st.binned_faces)
        info["pixel_tests"] = float(st.pixel_tests)
    return info


def kernel_bytes(kname, info, visible):
    """Algorithmic bytes one launch of `kname` must move: inputs read once,
    outputs written once; re-reads served by caches are not counted.
    F faces, P pixels, E bin entries, T tiles, B binned faces (those with a
    tile, listed for the scatter), V faces visible in the main
    pass (the front-most kept face of a pixel: with layered choosers a lower
    bound), vs varyings per corner, S chooser slots written per pixel."""
    F, P, E, T, vs = info["F"], info["P"], info["E"], info["T"], info["vs"]
    S = info.get("slots", 1)
    V = float(visible) if info["main"] else 0.0
    out_px = 16 if info["main"] else 4  # zbuffer (+ canvas) written
    table = {
        # plain form
        "vertex_kernel": info["cin"] + info["corners"] * (16 + 4 * vs),
        "setup_kernel": F * (12 + 3 * 16 + 64),
        "scan_kernel": F * 48 + P * 4 * S,
        "shade_kernel": P * (4 * S + out_px) + info["Ptex"] + V * (64 + 3 * (16 + 4 * vs)),
        # tiled form
        "setup_bin_kernel": F * (12 + 36 + 64 + 8) + info.get("B", 0.0) * 16 + E * 4,
        "scan_kernels": T * 12,
        "scatter_kernel": info.get("B", 0.0) * 16 + E * 12,
        "raster_kernel": F * 48 + E * 4 + P * 4 * S,
        "face_varyings_kernel": F + V * (12 + 3 * (info["cin"] / max(info["corners"], 1)) + 3 * 4 * vs),
        "tiled_shade_kernel": P * (4 * S + out_px) + info["Ptex"] + V * (64 + 3 * 4 * vs),
    }
    return table.get(kname, 0.0)


# The sources the tiled forward kernels are built from: the ncu counts below
# describe these kernels only while these files are unchanged.
FORWARD_SOURCES = ("jaxrenderer_gb300/csrc/rast_tiled.cu", "jaxrenderer_gb300/csrc/rast_internal.cuh",
                   "jaxrenderer_gb300/csrc/rast_math.cuh", "jaxrenderer_gb300/csrc/rast_shaders.cuh",
                   "include/rast_gb300.h")


def library_digest(files=FORWARD_SOURCES) -> str:
    """SHA-256 (16 hex digits) of the given CUDA sources (names and bytes)."""
    import hashlib

    h = hashlib.sha256()
    for name in files:
        p = ROOT / name
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()[:16]


# library_digest() of the sources the NCU_* counts below were captured on:
# when the kernels change, the counts no longer describe them and the bench
# reports traffic and the issue figure as null until they are captured again.
NCU_SOURCE_DIGEST = "d4e29622dd43f128"


def ncu_counts_current() -> bool:
    return library_digest() == NCU_SOURCE_DIGEST


# Per-unit counts of the forward kernels measured by ncu on the 256-scene
# brax-like batch with tile configs pinned (shadow 16x16 with two warps per
# tile, main 16x8: the autotuner's choice for the 4096-scene batch; and
# shadow 16x8 / main 8x8 for the raster's other entries): DRAM bytes
# (dram__bytes_read.sum + dram__bytes_write.sum) and warp instructions
# (smsp__inst_executed.sum) per face (F, 1,470,504 per pass) or per pixel of
# the pass (P: 1,806,336 main, 4,194,304 shadow).  Both grow with the faces or
# pixels a launch processes, so a full launch's are these times its units.
# Keyed by (pass, kernel); the raster kernel's also by its tile shape and
# warps per tile.
NCU_PER_UNIT = {
    ("shadow", "setup_bin_kernel"): ("F", 97.04, 25.07),
    ("main", "setup_bin_kernel"): ("F", 103.53, 26.49),
    ("shadow", "scatter_kernel"): ("F", 1.69, 1.56),
    ("main", "scatter_kernel"): ("F", 6.74, 3.97),
    ("shadow", "raster_kernel", 16, 16, 2): ("P", 3.15, 11.62),
    ("shadow", "raster_kernel", 16, 8, 1): ("P", 3.40, 11.68),
    ("main", "raster_kernel", 16, 8, 1): ("P", 29.32, 16.66),
    ("main", "raster_kernel", 8, 8, 1): ("P", 29.22, 19.56),
    ("main", "face_varyings_kernel"): ("F", 29.90, 4.60),
    ("main", "tiled_shade_kernel"): ("P", 59.80, 31.21),
}


def ncu_per_unit(pass_name, kname, cfg):
    """(unit, DRAM bytes per unit, warp instructions per unit) measured for
    this kernel on this pass (and tile config), or None."""
    if kname == "raster_kernel":
        if cfg is None:
            return None
        return NCU_PER_UNIT.get((pass_name, kname, int(cfg.tile_w), int(cfg.tile_h),
                                 max(int(getattr(cfg, "warps_per_tile", 1)), 1)))
    return NCU_PER_UNIT.get((pass_name, kname))


def issue_roofline(ms, clocks, warp_instr, source):
    """Issue-slot ceiling of a launch: `warp_instr` warp instructions per
    second of the live launch time, over SMs x 4 schedulers x the median SM
    clock sampled during the run."""
    import torch

    if ms <= 0 or warp_instr is None:
        return None
    mhz = (clocks or {}).get("sm_mhz") or (clocks or {}).get("sm_max_mhz")
    if not mhz:
        return None
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    peak = sms * 4 * float(mhz) * 1e6
    achieved = warp_instr / (ms / 1e3)
    return {"achieved": achieved, "peak": peak, "unit": "warp instructions/s", "frac": achieved / peak,
            "note": f"{source}; peak {sms} SMs x 4 schedulers x {float(mhz):.0f} MHz"}


def roofline(prof, visible, clocks=None):
    """HBM roofline of the dominant kernel: algorithmic bytes per launch /
    average launch duration (CUDA events inside the library); with the
    issue-slot figure beside it where ncu's instruction counts apply."""
    peak, kind = measured_peaks()
    summ = prof["summary"]
    infos = {}
    vis_of = {}
    runners = []
    for name, r, p in prof["passes"]:
        if r not in runners:
            runners.append(r)
    for r, v in zip(runners, visible):
        vis_of[id(r)] = v

    def bytes_of(name):
        r, p, kn = prof["where"][name]
        if (id(r), p) not in infos:
            infos[(id(r), p)] = pass_info(r, p)
        return kernel_bytes(kn, infos[(id(r), p)], vis_of.get(id(r), 0)), infos[(id(r), p)]

    cands = [n for n in summ if not n.endswith(":memset")]
    dom = max(cands, key=lambda k: summ[k]["avg_ms"])
    ms = summ[dom]["avg_ms"]
    alg, info = bytes_of(dom)
    achieved = alg / (ms / 1e3) / 1e9 if ms > 0 else 0.0
    per_kernel = {}
    current = ncu_counts_current()
    for name in cands:
        b, inf = bytes_of(name)
        v = summ[name]
        gbs = b / (v["avg_ms"] / 1e3) / 1e9 if v["avg_ms"] > 0 else None
        per_kernel[name] = {"bytes": b, "GB/s": gbs, "frac": gbs / peak if gbs is not None else None}
        r_k, p_k, k_k = prof["where"][name]
        c_k = r_k.configs.get(p_k)
        per_k = ncu_per_unit(p_k, k_k, c_k) if current and inf["slots"] == 1 and not (
            c_k is not None and int(c_k.small_area) > 0) else None
        if per_k is not None:
            per_kernel[name]["traffic"] = per_k[1] * inf[per_k[0]]
            iss = issue_roofline(v["avg_ms"], clocks, per_k[2] * inf[per_k[0]], "ncu per-unit count")
            per_kernel[name]["issue_frac"] = iss["frac"] if iss else None
    traffic, traffic_note, issue = None, None, None
    r_dom, p_dom, k_dom = prof["where"][dom]
    cfg = r_dom.configs.get(p_dom)
    small = cfg is not None and int(cfg.small_area) > 0
    per = ncu_per_unit(p_dom, k_dom, cfg)
    if not ncu_counts_current():
        traffic_note = (f"null: the kernels changed since the ncu capture the per-unit counts come from "
                        f"(sources {library_digest()}, capture {NCU_SOURCE_DIGEST})")
    elif per is None or small or info["slots"] != 1:
        traffic_note = "null: no ncu count for this kernel, pass and configuration"
    else:
        unit, bytes_per, instr_per = per
        units = info[unit]
        what = "face" if unit == "F" else "pixel"
        traffic = bytes_per * units
        traffic_note = (f"ncu DRAM bytes per {what} of this kernel and pass on the 256-scene brax-like case "
                        f"(same tile config) x this launch's {int(units)} {what}s")
        issue = issue_roofline(ms, clocks, instr_per * units,
                               f"ncu warp instructions per {what} on the 256-scene case x this launch's {what}s")
    out = {
        "bound": "hbm",
        "limiter": "hbm",
        "kernel": dom,
        "achieved": achieved,
        "peak": peak,
        "peak_source": kind,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": traffic,
        "traffic_note": traffic_note,
        "ncu_counts_digest": NCU_SOURCE_DIGEST,
        "algorithmic_bytes_per_launch": alg,
        "avg_launch_ms": ms,
    }
    if issue is not None:
        out["issue"] = issue
    issue = out.get("issue")
    if issue is not None and issue["frac"] > out["frac"]:
        out["limiter"] = "issue"  # instruction issue, not DRAM bandwidth, bounds this kernel (frac in "issue")
    kname = prof["where"][dom][2]
    if kname in ("scan_kernel", "raster_kernel"):
        tests = info["tests"] if kname == "scan_kernel" else info.get("pixel_tests")
        out["coverage"] = {"pixel_triangle_tests_per_s": tests / (ms / 1e3) if tests else None,
                           "pixel_triangle_tests_per_launch": tests or None,
                           "bin_entries": info["E"] or None,
                           "counted": ("W x H x F of the pass" if kname == "scan_kernel" else
                                       "in the kernel: dense entries x the warp's pixels + pair-path pairs, one add per warp")}
    return out, per_kernel


def measure_e2e(wl: Workload, mr, step, args, dev, stream, total_frames):
    """Public-API path with host inputs, all inside the timed region:
    instanced workloads copy the objects' transforms and scalings (pinned
    host -> device), rebuild the per-corner pools with rast_merge_objects and
    render; the others copy every per-corner input pool and render; then
    the canvases go to pinned host memory."""
    import torch

    host, outs = [], []
    h2d = d2h = 0
    if wl.merges:
        inst = wl.instances
        tr = torch.from_numpy(np.ascontiguousarray(inst.transforms)).pin_memory()
        sc = torch.from_numpy(np.ascontiguousarray(inst.local_scaling)).pin_memory()
        h2d = tr.numel() * 4 + sc.numel() * 4
    else:
        for r in mr.runners:
            hp = {}
            for n in INPUT_POOLS:
                if n not in r.sb.pools:
                    continue
                t = r.sb.pools[n]
                h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                h.copy_(t)
                hp[n] = h
                h2d += h.numel() * h.element_size()
            host.append(hp)
    results = [wl.display] if wl.notebook else [r.canvas for r in mr.runners]
    # two pinned host copies and two device staging copies of the results:
    # step k's device -> host copy runs on a copy stream while step k + 1
    # renders (pipelined serving); every copy finishes inside the timed region
    staging = [[torch.empty_like(t) for t in results] for _ in range(2)]
    for _ in range(2):
        outs.append([torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in results])
    d2h = sum(t.numel() * t.element_size() for t in results)
    copy_stream = torch.cuda.Stream(dev)
    copied = [None, None]  # event: staging[k] free again (its host copy done)
    rendered = [torch.cuda.Event(), torch.cuda.Event()]
    counter = [0]

    def e2e_step():
        k = counter[0] % 2
        counter[0] += 1
        if wl.notebook:  # the step itself merges
            wl.merges[0].transforms.copy_(tr.reshape(-1, 16), non_blocking=True)
            wl.merges[0].local_scaling.copy_(sc.reshape(-1, 3), non_blocking=True)
        elif wl.merges:
            wl.merges[0].merge(tr, sc, stream)
        for r, hp in zip(mr.runners, host):
            for n, h in hp.items():
                r.sb.pools[n].copy_(h, non_blocking=True)
        step()
        if copied[k] is not None:
            stream.wait_event(copied[k])
        for t, st in zip(results, staging[k]):
            st.copy_(t, non_blocking=True)
        rendered[k].record(stream)
        copy_stream.wait_event(rendered[k])
        with torch.cuda.stream(copy_stream):
            for st, oh in zip(staging[k], outs[k]):
                oh.copy_(st, non_blocking=True)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(copy_stream)
        copied[k] = ev

    # a pipelined loop's first and last frames overlap nothing: time enough
    # frames that they do not dominate.  Three trials of `steps` frames, the
    # median reported (a host-side stall of the shared box can hold one trial
    # back by several milliseconds); every trial's time is in the record.
    steps, trials = 20, 3
    trial_ms = []
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if wl.pipeline is not None and not wl.notebook:
        # instanced serving through batch.InstancedPipeline: frame k + 1's
        # transform copy and device merge overlap frame k's render, frame k's
        # canvases go to pinned host memory while frame k + 1 renders
        del staging
        torch.cuda.empty_cache()
        pipe = wl.pipeline()
        results = [pipe.canvas(0)]
        for k in range(4):  # warm-up frames (both sets, both host buffers)
            pipe.frame(tr, sc, out=outs[k % 2][0])
        pipe.synchronize()
        for _ in range(trials):
            torch.cuda.synchronize(dev)
            start.record(stream)
            pipe.start_after(start)
            for k in range(steps):
                pipe.frame(tr, sc, out=outs[k % 2][0])
            for ev in pipe.pending():  # the last copies end inside the timed region
                stream.wait_event(ev)
            stop.record(stream)
            torch.cuda.synchronize(dev)
            trial_ms.append(start.elapsed_time(stop) / steps)
        del pipe
    else:
        for _ in range(2):  # both staging and host buffers once
            e2e_step()
        torch.cuda.synchronize(dev)
        for _ in range(trials):
            torch.cuda.synchronize(dev)
            start.record(stream)
            for _ in range(steps):
                e2e_step()
            for ev in copied:  # the last copies end inside the timed region
                if ev is not None:
                    stream.wait_event(ev)
            stop.record(stream)
            torch.cuda.synchronize(dev)
            trial_ms.append(start.elapsed_time(stop) / steps)
    ms = float(np.median(trial_ms))
    out = {"value": total_frames / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
           "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": steps,
           "trials_ms_per_step": trial_ms,
           "inputs": ("object transforms + local scalings; per-corner pools rebuilt on the device "
                      "(rast_merge_objects)") if wl.merges else "per-corner input pools",
           "outputs": "uint8 display images" if wl.notebook else "float32 canvases",
           "pipelined": ("batch.InstancedPipeline: step k+1's transform copy and device merge on a merge stream "
                         "and step k's device->host copy on a copy stream, both overlapping the renders "
                         "(double-buffered pools and canvases)") if (wl.pipeline is not None and not wl.notebook)
                        else "device->host copy of step k on a copy stream overlapping step k+1"}
    if wl.merges:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            wl.merges[0].merge(stream=stream)
        b.record(stream)
        torch.cuda.synchronize(dev)
        out["device_merge_ms"] = a.elapsed_time(b) / steps
    out["link"] = copy_rates(dev, h2d, d2h)
    return out


def copy_rates(dev, h2d_bytes: int, d2h_bytes: int, reps: int = 3):
    """Host <-> device copy rates of one step's bytes, pinned host memory,
    one cudaMemcpyAsync each way on an idle stream (outside the timed
    region): what the e2e step's copies cost on this machine's link."""
    import torch

    out = {}
    s = torch.cuda.Stream(dev)
    for name, nbytes in (("h2d", h2d_bytes), ("d2h", d2h_bytes)):
        if nbytes <= 0:
            continue
        host = torch.empty(int(nbytes), dtype=torch.uint8, pin_memory=True)
        devbuf = torch.empty(int(nbytes), dtype=torch.uint8, device=dev)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(s):
            (devbuf.copy_(host, non_blocking=True) if name == "h2d" else host.copy_(devbuf, non_blocking=True))
            a.record(s)
            for _ in range(reps):
                (devbuf.copy_(host, non_blocking=True) if name == "h2d" else host.copy_(devbuf, non_blocking=True))
            b.record(s)
        torch.cuda.synchronize(dev)
        ms = a.elapsed_time(b) / reps
        out[f"{name}_gbs"] = nbytes / (ms / 1e3) / 1e9
        out[f"{name}_ms_per_step"] = ms
        del host, devbuf
    return out


# ------------------------------------------------------------- reference arm

def run_reference(args, rank, world, local):
    if rank != 0:
        return
    n = args.scenes
    if args.workload == "brax84":
        n = min(n, 256)  # scenes the sample draws from (the workload's first 256)
    wl = BUILDERS[args.workload](n, 0, None)
    wl.frames = args.scenes
    if len(wl.work) != args.scenes:
        wl.work = np.resize(wl.work, args.scenes)
    threads = len(os.sched_getaffinity(0))
    per_step = []
    budget = 6.0
    start = 0
    for k in range(args.warmup + args.steps):
        fps, done, el = oracle_rate(wl, budget, threads, start)
        start += done
        if k >= args.warmup:
            per_step.append((fps, done, el))
    value = float(np.mean([p[0] for p in per_step]))
    frames = sum(p[1] for p in per_step)
    secs = sum(p[2] for p in per_step)
    crop = f", main pass cropped to 1/{wl.oracle_crop} of the columns" if wl.oracle_crop > 1 else ""
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "impl": "reference",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs / len(per_step) * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": wl.data,
        "config": dict({"workload": wl.desc, "sample_per_step": f"~{budget:.0f} s of consecutive scenes{crop}"},
                       **wl.config),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{frames} scenes over {len(per_step)} steps; JAX is not installable, so the "
                                   "CPU path timed is the C restatement of the reference (oracle/)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def launch_ranks(n: int) -> int:
    """`--gpus N` outside a launcher: start one process per GPU as
    `python -m torch.distributed.run --nnodes=1 --nproc-per-node N` would
    (rendezvous on 127.0.0.1) and return their exit status."""
    import socket

    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", str(Path(__file__).resolve()), *sys.argv[1:]]
    return subprocess.call(cmd)


def main():
    args = parse()
    rank, world, local = dist_env()
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        sys.exit(launch_ranks(args.gpus))
    if world != args.gpus:
        print(json.dumps({"error": f"--gpus {args.gpus} but {world} ranks were launched"}), flush=True)
        sys.exit(2)
    if args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
