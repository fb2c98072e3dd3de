"""Autotuner of the tiled form: tile shape, small-face path, warps per
tile and bin capacity per workload.

The search itself is the library's rast_autotune (C ABI): every tile shape
with a kernel (8x8, 16x8, 16x16, 32x8, 8x32, 8x4 and 4x8 with one warp per
tile; 8x8, 8x16 and 16x16 with two warps each taking half of the rows; the
layered shapes for passes with layered-chooser jobs), with the setup
kernel's small-face rasterisation off and on, is timed on the batch itself
with a bin capacity of 1.25x the entries its shape requests, and the
fastest wins.  The library caches results per process; this module keeps
them across processes in a JSON file keyed by (width, height, faces-per-job
bucket, jobs bucket, shader mask, layers, device name, SM count), so a
workload class is tuned once per machine.
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

SHAPES = ((8, 8), (16, 8), (16, 16), (32, 8), (8, 32), (8, 4), (4, 8))  # one warp per tile
TWO_WARP_SHAPES = ((8, 8), (8, 16), (16, 16))  # two warps per tile, half of the rows each
LAYERED_SHAPES = ((8, 8), (16, 8), (8, 4), (4, 8))  # one-warp shapes with a layered-chooser raster variant
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
    return (f"v4|{w}x{h}|f~{bucket}|jobs~{2 ** int(round(math.log2(max(len(jobs), 1))))}|mask{mask}"
            + (f"|layers{layers}" if layers > 0 else "") + f"|{props.name}|sm{props.multi_processor_count}")


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
                                    int(hit.get("small_area", 0)), int(hit.get("warps_per_tile", 1)))
    cfg = _lib.RastTiledConfig()
    with torch.cuda.device(device):
        s = torch.cuda.current_stream(device)
        _lib.check(_lib.load().rast_autotune(ctypes.byref(b), s.cuda_stream, ctypes.byref(cfg)), "rast_autotune")
    with _LOCK:
        cache = _load()
        cache[key] = {"tile_w": cfg.tile_w, "tile_h": cfg.tile_h, "bin_capacity": int(cfg.bin_capacity),
                      "small_area": cfg.small_area, "warps_per_tile": cfg.warps_per_tile}
        _store(cache)
    return cfg


__all__ = ["tiled_config_for", "tiled_config_for_batch", "workload_key", "cache_path", "SHAPES", "TWO_WARP_SHAPES",
           "LAYERED_SHAPES", "SMALL_AREAS"]
