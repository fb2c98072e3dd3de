"""Masked central differences of the FP64 oracle, for checking the CUDA
backward (rast_backward) on full-size scenes.

The loss is L = sum over pixels p in M and channels of
(canvas_p - target_p)^2 / N, N = W * H * 3 (a mean squared error).  M is the
set of pixels the base render writes whose winning primitive and fragment
branch signature (sampled texel, the shader's lighting / keep branches; see
oracle/rast_oracle.h) stay the same in every perturbed render: on M the
canvas is a smooth function of every input checked, which is the piecewise-
constant visibility of jax.grad on the reference.  Every coordinate is
evaluated at x +- eps and x +- eps / 2 (eps = 1e-3, FP64):

  g     = (L(x + eps) - L(x - eps)) / (2 eps)          the checked value
  tau   = 4/3 |g - g_half|                             its truncation error
                                                       (Richardson estimate)
  S     = sum_p |per-pixel loss differences| / (2 eps) the scale of the terms
                                                       the gradient sums

and the analytic gradient g_an passes when both

  |g_an - g|   <= RTOL |g| + 2 tau + 1e-5 S,          RTOL = 1e-3,
  |g_an - g_R| <= RTOL |g_R| + 1e-5 S,   g_R = (4 g_half - g) / 3.

The floor 2 tau covers the FD's own O(eps^2) error (on the small triangles
of a level-4 sphere the eps = 1e-3 FD of a vertex coordinate is off by up
to a few percent); g_R, the Richardson extrapolation, has no eps^2 term
and needs no such floor.  1e-5 S covers FP32 rounding of the analytic
terms (a few tens of roundings of 2^-24 each per term, summed with
cancellation).

A coordinate may carry a pixel window: only pixels whose base winner
depends on that coordinate can change (faces incident to a vertex, pixels
sampling a texel), so the oracle renders just that window.  Pixels outside
it contribute zero to both sides.

Test infrastructure only.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Sequence, Tuple

import numpy as np

EPS = 1e-3
RTOL = 1e-3
FP32_FLOOR = 1e-5

Window = Optional[Tuple[int, int, int, int]]


@dataclass
class Coord:
    tensor: str
    index: int  # flat index into the tensor
    window: Window = None


@dataclass
class FDResult:
    coord: Coord
    g: float
    g_half: float
    scale: float

    @property
    def richardson(self) -> float:
        """(4 g_half - g) / 3: the FD with its eps^2 term cancelled."""
        return (4.0 * self.g_half - self.g) / 3.0

    @property
    def tau(self) -> float:
        return 4.0 / 3.0 * abs(self.g - self.g_half)

    def bound(self) -> float:
        return RTOL * abs(self.g) + 2.0 * self.tau + FP32_FLOOR * self.scale


def _slices(window: Window, W: int, H: int):
    if window is None:
        return slice(0, W), slice(0, H)
    return slice(window[0], window[1]), slice(window[2], window[3])


def pixel_window(mask: np.ndarray, pad: int = 2) -> Window:
    """Bounding box (x0, x1, y0, y1) of the True pixels of `mask`, widened by
    `pad` and clipped to the buffer; None when the mask is empty."""
    ij = np.argwhere(mask)
    if ij.size == 0:
        return None
    W, H = mask.shape
    x0, y0 = ij.min(0) - pad
    x1, y1 = ij.max(0) + 1 + pad
    return (max(int(x0), 0), min(int(x1), W), max(int(y0), 0), min(int(y1), H))


def vertex_windows(faces: np.ndarray, prim: np.ndarray, verts: Sequence[int], pad: int = 2) -> Dict[int, Window]:
    """Window of each vertex: the pixels whose base winner is one of the
    faces that use the vertex."""
    out = {}
    for v in verts:
        incident = np.nonzero((faces == v).any(1))[0]
        out[int(v)] = pixel_window(np.isin(prim, incident), pad)
    return out


def texel_windows(texel: np.ndarray, rows: Sequence[int], pad: int = 1) -> Dict[int, Window]:
    """Window of each texel row: the pixels that sampled it."""
    return {int(t): pixel_window(texel == t, pad) for t in rows}


def masked_fd(render: Callable[[Dict[str, np.ndarray], Window], dict], x0: Dict[str, np.ndarray],
              coords: Sequence[Coord], base: dict, target: np.ndarray) -> Tuple[np.ndarray, List[FDResult]]:
    """Central differences of the masked MSE for every coordinate.

    `render(params, window)` renders the FP64 oracle with `params` (a dict of
    float64 arrays, same keys as x0) inside `window` and returns its dict
    (canvas, prim_id, branch).  `base` is the unperturbed full render.
    Returns (M as a bool (W, H) array, one FDResult per coordinate)."""
    W, H = base["prim_id"].shape
    N = float(W * H * 3)
    changed = np.zeros((W, H), bool)
    renders = []
    for c in coords:
        sx, sy = _slices(c.window, W, H)
        canv = {}
        for h in (EPS, -EPS, 0.5 * EPS, -0.5 * EPS):
            x = dict(x0)
            a = np.array(x0[c.tensor], np.float64, copy=True)
            a.reshape(-1)[c.index] += h
            x[c.tensor] = a
            out = render(x, c.window)
            changed[sx, sy] |= (out["prim_id"][sx, sy] != base["prim_id"][sx, sy]) | (
                out["branch"][sx, sy] != base["branch"][sx, sy])
            canv[h] = out["canvas"][sx, sy]
        renders.append(canv)
    M = (base["prim_id"] >= 0) & ~changed
    results = []
    for c, canv in zip(coords, renders):
        sx, sy = _slices(c.window, W, H)
        m = M[sx, sy][..., None]
        t = target[sx, sy]

        def diff(h):
            return np.where(m, (canv[h] - t) ** 2 - (canv[-h] - t) ** 2, 0.0)

        d_full, d_half = diff(EPS), diff(0.5 * EPS)
        g = float(d_full.sum()) / (2 * EPS * N)
        g_half = float(d_half.sum()) / (EPS * N)
        scale = float(np.abs(d_full).sum()) / (2 * EPS * N)
        results.append(FDResult(c, g, g_half, scale))
    return M, results


def compare(results: Sequence[FDResult], analytic: Dict[str, np.ndarray]) -> Dict[str, dict]:
    """Check every coordinate; returns per-tensor statistics and raises
    AssertionError listing the coordinates outside their bound."""
    fails = []
    stats: Dict[str, dict] = {}
    for r in results:
        g_an = float(np.asarray(analytic[r.coord.tensor]).reshape(-1)[r.coord.index])
        err = abs(g_an - r.g)
        s = stats.setdefault(r.coord.tensor, {"n": 0, "nonzero": 0, "within_rtol": 0, "max_rel": 0.0,
                                              "max_rel_richardson": 0.0, "max_err_over_bound": 0.0})
        s["n"] += 1
        s["within_rtol"] += int(err <= RTOL * abs(r.g))
        if r.g != 0.0:
            s["nonzero"] += 1
            s["max_rel"] = max(s["max_rel"], err / abs(r.g))
            s["max_rel_richardson"] = max(s["max_rel_richardson"], abs(g_an - r.richardson) / abs(r.g))
        b = r.bound()
        s["max_err_over_bound"] = max(s["max_err_over_bound"], err / b if b > 0 else (0.0 if err == 0 else np.inf))
        if err > b:
            fails.append((r.coord.tensor, r.coord.index, g_an, r.g, r.tau, r.scale))
        # and against the extrapolated FD, whose eps^2 term is gone: no truncation floor
        err_r = abs(g_an - r.richardson)
        if err_r > RTOL * abs(r.richardson) + FP32_FLOOR * r.scale:
            fails.append(("richardson", r.coord.tensor, r.coord.index, g_an, r.richardson, r.scale))
    assert not fails, f"{len(fails)} coordinates outside rtol {RTOL}: {fails[:8]}"
    return stats
