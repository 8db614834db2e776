"""Helpers (sparrowpy/utils): geometry files through `utils.blender`."""
from . import blender

__all__ = ["blender"]
