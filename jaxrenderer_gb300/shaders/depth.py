"""DepthShader (renderer/shaders/depth.py:20-61): gl_Position only."""
from typing import Any, NamedTuple

from .. import _lib
from ..shader import Shader


class DepthExtraInput(NamedTuple):
    position: Any  # (vertices, 3) world space


class DepthExtraFragmentData(NamedTuple):
    pass


class DepthExtraMixerOutput(NamedTuple):
    pass


class DepthShader(Shader):
    """Depth only; no colour target."""

    kernel_id = _lib.SHADER_DEPTH
    extra_input = DepthExtraInput
