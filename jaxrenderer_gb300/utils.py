"""Display helpers (renderer/utils.py of jaxrenderer)."""
from __future__ import annotations

import numpy as np
import torch


def transpose_for_display(matrix, flip_vertical: bool = True):
    """Swap the first two axes ((W, H, ...) -> (H, W, ...)) and, by default,
    flip the new first axis so row 0 is the top (utils.py:79-96)."""
    if isinstance(matrix, torch.Tensor):
        mat = matrix.transpose(0, 1)
        return mat.flip(0) if flip_vertical else mat
    mat = np.swapaxes(np.asarray(matrix), 0, 1)
    return mat[::-1, ...] if flip_vertical else mat


def build_texture_from_PyTinyrenderer(texture, width: int, height: int) -> np.ndarray:
    """PyTinyrenderer's flat RGB buffer -> (width, height, channels) texture
    (utils.py:101-125)."""
    t = np.reshape(np.asarray(texture, dtype=np.float32), (width, height, -1), order="C")
    return np.ascontiguousarray(np.swapaxes(t, 0, 1)[:, ::-1, :])


__all__ = ["transpose_for_display", "build_texture_from_PyTinyrenderer", "display_u8"]


def display_u8(canvas, flip_vertical: bool = True, out=None, stream=None):
    """transpose_for_display((clamp(canvas, 0, 1) * 255).astype(uint8)) on
    the device (the notebooks' epilogue; rast_display_u8): canvas (W, H, C)
    or (N, W, H, C) float32 CUDA tensor -> (H, W, C) / (N, H, W, C) uint8."""
    from . import _lib

    single = canvas.dim() == 3
    c = canvas.contiguous()
    if single:
        c = c.unsqueeze(0)
    n, w, h, ch = c.shape
    if out is None:
        out = torch.empty((n, h, w, ch), dtype=torch.uint8, device=c.device)
    s = stream if stream is not None else torch.cuda.current_stream(c.device)
    lib = _lib.load()
    _lib.check(lib.rast_display_u8(c.data_ptr(), n, w, h, ch, int(bool(flip_vertical)), out.data_ptr(), s.cuda_stream),
               "rast_display_u8")
    return out[0] if single else out

