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


__all__ = ["transpose_for_display", "build_texture_from_PyTinyrenderer"]
