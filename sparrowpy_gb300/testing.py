"""Testing utilities (sparrowpy/testing/__init__.py): the shoebox room stub."""
from .geometry import shoebox_room_stub

__all__ = ["shoebox_room_stub"]
