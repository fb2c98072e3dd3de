"""Benchmark: frames/s of the rasterisation path at 84x84 x 4096 scenes.

Workload (the reference's Brax-style 84x84 benchmark, seeded synthetic
stand-in): 4096 scenes, each a ground plane plus 8-32 objects drawn from
{box 12 tris, icosphere level 2 320 tris, capsule 16x8 512 tris}, uneven
triangle counts (mean ~5.7k per scene), PhongReflectionShadowTextureShader
with a 128x128 light-space depth map.  One step renders every scene once:
the depth pass of all scenes, then the main pass of all scenes.  One frame is
one scene's final canvas.

    python bench.py [--steps K] [--warmup W] [--form plain|tiled] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is device-resident throughput; `e2e`
is the same work through the public batch API with the scene inputs copied
from pinned host memory and the canvases copied back inside the timed region.
`--impl reference` times the CPU oracle (the C restatement of the reference's
JAX path) on a bounded sample of the same workload, with all host threads.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "frames/s @84x84x4096 scenes fwd and fwd+bwd, tiled-batched vs plain GPU"
UNIT = "frames/s"
N_SCENES = 4096
W = H = 84
SHADOW = (128, 128)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--form", choices=["plain", "tiled", "auto"], default="auto")
    p.add_argument("--scenes", type=int, default=N_SCENES)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-plain", action="store_true")
    p.add_argument("--no-bwd", action="store_true")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------ CPU baseline

def _oracle_frame(flat, sb_tables, s, threads):
    from oracle import oracle

    dspec, mspec = sb_tables(s)
    smap = oracle.render(dspec, np.full(SHADOW, np.finfo(np.float32).max, np.float32), n_threads=threads)["zbuffer"]
    mspec.shadow_map = smap
    oracle.render(mspec, np.ones((W, H), np.float32), np.ones((W, H, 3), np.float32), n_threads=threads)


def time_oracle(flat, tables_fn, budget_s: float, threads: int):
    """Render consecutive scenes with the oracle until `budget_s` is spent."""
    done = 0
    t0 = time.perf_counter()
    while True:
        _oracle_frame(flat, tables_fn, done % flat.n_scenes, threads)
        done += 1
        el = time.perf_counter() - t0
        if el >= budget_s:
            return done, el


class HostTables:
    """Job tables of a FlatScenes batch without a device (for the oracle)."""

    def __init__(self, flat):
        from jaxrenderer_gb300 import batch as jb

        self.flat = flat
        self.tables = jb.scene_batch_tables(flat, W, H, shadow_size=SHADOW)

    def __call__(self, s):
        from jaxrenderer_gb300 import batch as jb

        return jb.scene_job_specs(self.flat, self.tables, s)


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
                                          "--format=csv,noheader,nounits", "-lms", "100"],
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

def run_ours(args, rank, world, local):
    import torch

    from jaxrenderer_gb300 import _lib, batch as jb, synthetic

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    _lib.load()
    form = "tiled" if args.form == "auto" else args.form
    flat = synthetic.brax_like_batch(args.scenes, seed=synthetic.BASE_SEED + 1 + rank)
    sb = jb.scene_batch_from_flat(flat, W, H, shadow_size=SHADOW, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    def timed(step_fn, steps, warmup, clocks=None):
        for _ in range(warmup):
            step_fn()
        barrier()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for _ in range(steps):
            step_fn()
        stop.record(stream)
        barrier()
        ms = start.elapsed_time(stop)
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms / steps

    runner = jb.BatchRunner(sb, form=form, want_prim_id=False)
    if form == "tiled":
        runner.capture()
        step = runner.replay
    else:
        step = lambda: runner.run(stream)  # noqa: E731
    for _ in range(args.warmup):
        step()
    with ClockSampler(local) as clk:
        ms_per_step = timed(step, args.steps, 0)
    value = world * args.scenes / (ms_per_step / 1e3)
    prof = profile_kernels(runner, args.steps, stream)

    comparison = {}
    if form == "tiled" and not args.no_plain:
        plain = jb.BatchRunner(sb, form="plain", want_prim_id=False)
        pms = timed(lambda: plain.run(stream), max(1, min(args.steps, 3)), 1)
        comparison = {"plain_fwd": world * args.scenes / (pms / 1e3), "plain_ms_per_step": pms,
                      "tiled_over_plain": pms / ms_per_step}
        del plain
        torch.cuda.empty_cache()

    fwd_bwd = {}
    if not args.no_bwd:
        fwd_bwd = measure_fwd_bwd(sb, args, stream, timed, world)

    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(flat, sb, runner, step, args, dev, stream, world)

    kernels_per_step = len(prof["per_step_names"])
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
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded Brax-like scenes; the reference's Brax fixtures are inputs-only pickles)",
        "config": {
            "workload": "brax-like 84x84 x 4096 scenes, phong_reflection_shadow + 128x128 depth pass",
            "form": form + (" (CUDA graph replay)" if form == "tiled" else ""),
            "tiled_config": {k: [c.tile_w, c.tile_h, int(c.bin_capacity)] for k, c in runner.configs.items()},
            "scenes": args.scenes,
            "mean_faces_per_scene": float(flat.n_faces.mean()),
            "resolution": [W, H],
            "shadow_map": list(SHADOW),
            "l2": "inputs larger than L2 (per-corner pools %.2f GB)" % (flat.position.nbytes * 3 / 1e9),
            "parallelism": f"scene-sharded x{world} (no collective)",
        },
        "fwd_comparison": comparison,
        "fwd_bwd": fwd_bwd,
        "roofline": roofline(prof, sb, flat, runner),
        "kernels": prof["summary"],
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": clk.summary(),
    }
    if e2e is not None:
        out["e2e"] = e2e
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_line(flat, budget_s=12.0)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def measure_fwd_bwd(sb, args, stream, timed, world):
    """Forward + backward of an MSE loss against a fixed target image, per
    step: render (prim-id buffer saved), dL/dcanvas, rast_backward into
    reused gradient arrays (per-vertex, per-texel, per-scene camera/light)."""
    import torch

    from jaxrenderer_gb300 import batch as jb

    out = {}
    target = torch.rand((sb.n_scenes, W, H, 3), generator=torch.Generator().manual_seed(0)).to(sb.device)
    scale = 2.0 / target.numel()
    for form in ("tiled", "plain"):
        if form == "plain" and args.no_plain:
            continue
        r = jb.BatchRunner(sb, form=form, want_prim_id=True)
        grads = r.grad_buffers()
        if form == "tiled":
            r.capture()
            fwd = r.replay
        else:
            fwd = lambda r=r: r.run(stream)  # noqa: E731

        def step(r=r, fwd=fwd, grads=grads):
            o = fwd()
            g = (o.canvas - target) * scale
            r.backward(g, out=grads)

        steps = args.steps if form == "tiled" else max(1, min(args.steps, 3))
        ms = timed(step, steps, 1 if form == "plain" else args.warmup)
        out[form] = {"value": world * args.scenes / (ms / 1e3), "ms_per_step": ms, "steps": steps}
        # backward alone, and its kernels (CUDA events inside the library)
        if form == "tiled":
            from jaxrenderer_gb300 import _lib

            fwd()
            gc = (r.canvas - target) * scale
            bms = timed(lambda: r.backward(gc, out=grads), steps, 1)
            out["backward_ms"] = bms
            prof = _lib.RastProfile()
            r.backward(gc, out=grads, profile=prof)
            out["backward_kernels_ms"] = {prof.names[k].decode(): prof.ms[k] for k in range(prof.n)}
        del r, grads
        torch.cuda.empty_cache()
    if "plain" in out:
        out["tiled_over_plain"] = out["plain"]["ms_per_step"] / out["tiled"]["ms_per_step"]
    out["unit"] = UNIT
    return out


def profile_kernels(runner, steps, stream):
    """Per-kernel CUDA-event durations inside the library, same steps again."""
    from jaxrenderer_gb300 import _lib

    acc = {}
    names_order = []
    for _ in range(steps):
        runner._reset(1.0)
        for key, _b in runner.batches():
            prof = _lib.RastProfile()
            runner.launch(key, stream.cuda_stream, profile=prof)
            for k in range(prof.n):
                name = f"{key}:{prof.names[k].decode()}"
                if name not in acc:
                    acc[name] = []
                    names_order.append(name)
                acc[name].append(prof.ms[k])
    summary = {n: {"avg_ms": float(np.mean(v)), "launches": len(v)} for n, v in acc.items()}
    total = sum(v["avg_ms"] for v in summary.values())
    for v in summary.values():
        v["share"] = v["avg_ms"] / total if total > 0 else 0.0
    return {"summary": summary, "per_step_names": names_order}


def _lib_profile():
    from jaxrenderer_gb300 import _lib

    return _lib.RastProfile()


def kernel_bytes(kname, pass_name, sb, flat, runner):
    """Algorithmic bytes one launch of `kname` must move (roofline):
    inputs read once, outputs written once; re-reads served by caches are
    not counted."""
    F = int(flat.n_faces.sum())
    corners = 3 * F
    main = pass_name == "main"
    pixels = sb.n_scenes * (W * H if main else SHADOW[0] * SHADOW[1])
    entries = 0
    if runner.form == "tiled":
        entries = int(runner.stats(pass_name).bin_entries)
    out_px = (4 + 12) if main else 4  # zbuffer (+ canvas) written
    table = {
        # plain form
        "vertex_kernel": corners * (12 + (12 + 8 + 4 if main else 0)) + corners * (16 + (40 if main else 0)),
        "setup_kernel": F * (12 + 3 * 16 + 64),
        "scan_kernel": F * 48 + pixels * 4,
        "shade_kernel": pixels * (4 + out_px + (4 if main else 0)),
        # tiled form
        "setup_bin_kernel": F * (12 + 36 + 64 + 8) + entries * 4,
        "scan_kernels": runner_tiles(runner, pass_name) * 12,
        "scatter_kernel": F * 8 + entries * 12,
        "raster_kernel": F * 48 + entries * 4 + pixels * 4,
        "tiled_shade_kernel": pixels * (4 + out_px + (4 if main else 0)),
    }
    return table.get(kname, 0), entries


def runner_tiles(runner, pass_name):
    if runner.form != "tiled":
        return 0
    return int(runner.stats(pass_name).tiles)


def roofline(prof, sb, flat, runner):
    """HBM roofline of the dominant kernel: algorithmic bytes per launch /
    average launch duration (CUDA events inside the library)."""
    peak, kind = measured_peaks()
    summ = prof["summary"]
    dom = max(summ, key=lambda k: summ[k]["avg_ms"])
    ms = summ[dom]["avg_ms"]
    pass_name, kname = dom.split(":")
    alg, entries = kernel_bytes(kname, pass_name, sb, flat, runner)
    achieved = alg / (ms / 1e3) / 1e9 if ms > 0 else 0.0
    pixels = sb.n_scenes * (W * H if pass_name == "main" else SHADOW[0] * SHADOW[1])
    per_kernel = {}
    for name, v in summ.items():
        pn, kn = name.split(":")
        b, _ = kernel_bytes(kn, pn, sb, flat, runner)
        per_kernel[name] = {"GB/s": b / (v["avg_ms"] / 1e3) / 1e9 if v["avg_ms"] > 0 else None,
                            "frac": (b / (v["avg_ms"] / 1e3) / 1e9) / peak if v["avg_ms"] > 0 else None}
    out = {
        "bound": "hbm",
        "kernel": dom,
        "achieved": achieved,
        "peak": peak,
        "peak_source": kind,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": None,
        "algorithmic_bytes_per_launch": alg,
        "avg_launch_ms": ms,
        "per_kernel": per_kernel,
    }
    if kname in ("scan_kernel", "raster_kernel"):
        tests = pixels * float(flat.n_faces.mean()) if kname == "scan_kernel" else None
        out["coverage"] = {"pixel_triangle_tests_per_s": tests / (ms / 1e3) if tests else None,
                           "bin_entries": entries or None,
                           "note": "coverage is FP32-issue bound; issue-slot utilisation in profiles/"}
    return out


def measure_e2e(flat, sb, runner, step, args, dev, stream, world):
    """Public-API path with host inputs: pinned host pools -> device, render,
    canvases -> pinned host, all inside the timed region."""
    import torch

    names = ["position", "normal", "uv", "texture_index", "texture", "specular_map"]
    host = {}
    for n in names:
        t = sb.pools[n]
        h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
        h.copy_(t)
        host[n] = h
    out_host = torch.empty(runner.canvas.shape, dtype=torch.float32, pin_memory=True)
    h2d = sum(host[n].numel() * host[n].element_size() for n in names)
    d2h = out_host.numel() * 4

    def e2e_step():
        for n in names:
            sb.pools[n].copy_(host[n], non_blocking=True)
        step()
        out_host.copy_(runner.canvas, non_blocking=True)

    steps = max(1, min(args.steps, 5))
    e2e_step()
    torch.cuda.synchronize(dev)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        e2e_step()
    stop.record(stream)
    torch.cuda.synchronize(dev)
    ms = start.elapsed_time(stop) / steps
    return {"value": world * args.scenes / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "steps": steps}


def cpu_baseline_line(flat, budget_s: float):
    threads = len(os.sched_getaffinity(0))
    tables = HostTables(flat)
    _oracle_frame(flat, tables, 0, threads)  # build + warm
    done, el = time_oracle(flat, tables, budget_s, threads)
    return {"value": done / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{done} consecutive scenes of the workload (depth + main pass each), oracle C restatement, "
                      f"OpenMP over pixel columns, {el:.1f} s"}


# ------------------------------------------------------------- reference arm

def run_reference(args, rank, world, local):
    if rank != 0:
        return
    from jaxrenderer_gb300 import synthetic

    flat = synthetic.brax_like_batch(min(args.scenes, 256), seed=synthetic.BASE_SEED + 1)
    threads = len(os.sched_getaffinity(0))
    tables = HostTables(flat)
    _oracle_frame(flat, tables, 0, threads)
    per_step = []
    budget = 6.0
    for k in range(args.warmup + args.steps):
        done, el = time_oracle(flat, tables, budget, threads)
        if k >= args.warmup:
            per_step.append((done, el))
    frames = sum(d for d, _ in per_step)
    secs = sum(e for _, e in per_step)
    value = frames / secs
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
        "data": "synthetic (seeded Brax-like scenes)",
        "config": {"workload": "brax-like 84x84 x 4096 scenes, phong_reflection_shadow + 128x128 depth pass",
                   "sample_per_step": f"~{budget:.0f} s of consecutive scenes"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{frames} scenes over {len(per_step)} steps; JAX is not installable, so the "
                                   "CPU path timed is the C restatement of the reference (oracle/)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world, local)
    else:
        run_ours(args, rank, world, local)


if __name__ == "__main__":
    main()
