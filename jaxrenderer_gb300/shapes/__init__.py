"""Procedural meshes: `create_cube` and `create_capsule`."""
from .capsule import UpAxis, create_capsule
from .cube import create_cube

__all__ = ["UpAxis", "create_capsule", "create_cube"]
