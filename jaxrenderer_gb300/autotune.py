"""Autotuner of the tiled form: tile shape, small-face path and bin
capacity per workload.

For a pass (one RastBatch) the tile shapes 8x8, 16x8, 16x16, 32x8, 8x32,
8x4 and 4x8 (pixels along x by y), each with the setup kernel's small-face
rasterisation off and on, are timed on the batch itself; the fastest wins.
Passes with layered-chooser jobs try the four shapes that have a layered
raster variant, without the small-face path.
The bin capacity is then set to 1.25x the bin entries that shape requested.
Results are cached in a JSON file keyed by (width, height, faces-per-job
bucket, shader mask, device name, SM count), so a workload class is tuned
once per machine.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
import threading
from pathlib import Path

import numpy as np
import torch

from . import _lib

SHAPES = ((8, 8), (16, 8), (16, 16), (32, 8), (8, 32), (8, 4), (4, 8))
LAYERED_SHAPES = ((8, 8), (16, 8), (8, 4), (4, 8))  # shapes with a layered-chooser raster variant
SMALL_AREAS = (0, 32)  # small-face rasterisation in the setup kernel: off, or rectangles up to 32 pixels
_LOCK = threading.Lock()


def cache_path() -> Path:
    env = os.environ.get("JAXRENDERER_GB300_AUTOTUNE")
    if env:
        return Path(env)
    return Path(__file__).resolve().parent / "_build" / "autotune.json"


def _load() -> dict:
    p = cache_path()
    if p.exists():
        try:
            return json.loads(p.read_text())
        except (OSError, ValueError):
            return {}
    return {}


def _store(d: dict) -> None:
    p = cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    tmp = p.with_suffix(".tmp")
    tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
    os.replace(tmp, p)


def workload_key(jobs: np.ndarray, device: torch.device) -> str:
    props = torch.cuda.get_device_properties(device)
    w, h = int(jobs["width"].max()), int(jobs["height"].max())
    f = float(jobs["n_faces"].mean())
    bucket = 2 ** int(round(math.log2(max(f, 1.0))))
    mask = int(np.bitwise_or.reduce(1 << jobs["shader"].astype(np.int64)))
    layers = int(jobs["layers"].max())
    return (f"v3|{w}x{h}|f~{bucket}|jobs~{2 ** int(round(math.log2(max(len(jobs), 1))))}|mask{mask}"
            + (f"|layers{layers}" if layers > 0 else "") + f"|{props.name}|sm{props.multi_processor_count}")


def _time(dev, b, cfg, reps=3) -> float:
    lib = _lib.load()
    nbytes = int(lib.rast_tiled_workspace_bytes(ctypes.byref(b), ctypes.byref(cfg)))
    ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev)
    s = torch.cuda.current_stream(dev)
    st = lib.rast_render_tiled(ctypes.byref(b), ctypes.byref(cfg), ws.data_ptr(), nbytes, s.cuda_stream)
    _lib.check(st, "autotune warm-up")
    stats = _lib.RastTiledStats()
    _lib.check(lib.rast_tiled_stats(ctypes.byref(b), ctypes.byref(cfg), ws.data_ptr(), s.cuda_stream,
                                    ctypes.byref(stats)), "autotune stats")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        lib.rast_render_tiled(ctypes.byref(b), ctypes.byref(cfg), ws.data_ptr(), nbytes, s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize(dev)
    return e0.elapsed_time(e1) / reps, int(stats.bin_entries)


def tiled_config_for(runner, name: str, b, jobs: np.ndarray) -> "_lib.RastTiledConfig":
    """Tuned RastTiledConfig for one pass of a BatchRunner."""
    return tiled_config_for_batch(runner.sb.device, b, jobs)


def tiled_config_for_batch(device: torch.device, b, jobs: np.ndarray) -> "_lib.RastTiledConfig":
    """Tuned RastTiledConfig for a RastBatch `b` whose job table is `jobs`
    (structured array with the RastJob layout).  Tuning renders `b` several
    times into its own output pools: pass a batch whose outputs may be
    overwritten."""
    key = workload_key(jobs, device)
    with _LOCK:
        cache = _load()
        hit = cache.get(key)
    if hit is not None:
        return _lib.RastTiledConfig(int(hit["tile_w"]), int(hit["tile_h"]), int(hit["bin_capacity"]),
                                    int(hit.get("small_area", 0)))
    best = None
    layered = int(jobs["layers"].max()) > 0  # no small-face path and fewer shapes
    for tw, th in LAYERED_SHAPES if layered else SHAPES:
        for small in (0,) if layered else SMALL_AREAS:
            cfg = _lib.RastTiledConfig(tw, th, 0, small)
            ms, entries = _time(device, b, cfg)
            if best is None or ms < best[0]:
                best = (ms, tw, th, entries, small)
    ms, tw, th, entries, small = best
    cap = int(entries * 1.25) + 4096
    with _LOCK:
        cache = _load()
        cache[key] = {"tile_w": tw, "tile_h": th, "bin_capacity": cap, "small_area": small, "ms": ms}
        _store(cache)
    return _lib.RastTiledConfig(tw, th, cap, small)


__all__ = ["tiled_config_for", "tiled_config_for_batch", "workload_key", "cache_path", "SHAPES", "LAYERED_SHAPES", "SMALL_AREAS"]
