"""GouraudShader (renderer/shaders/gouraud.py:49-124)."""
from typing import Any, NamedTuple

from .. import _lib
from ..shader import Shader
from ..types import LightSource


class GouraudExtraInput(NamedTuple):
    position: Any  # (vertices, 3) world space
    colour: Any  # (vertices, 3)
    normal: Any  # (vertices, 3) world space
    light: LightSource


class GouraudExtraFragmentData(NamedTuple):
    colour: Any = (0.0, 0.0, 0.0)


class GouraudExtraMixerOutput(NamedTuple):
    canvas: Any


class GouraudShader(Shader):
    """Per-vertex lighting, interpolated colour; fragments with a negative
    channel are discarded."""

    kernel_id = _lib.SHADER_GOURAUD
    extra_input = GouraudExtraInput
