"""Geometry files (sparrowpy/utils/blender.py:22-97) without Blender.

`read_geometry_file` reads .blend and .stl files into the fine and rough
meshes the reference returns (sparrowpy_gb300.mesh).  The Blender-session
helpers of the reference (ensure_object_mode, generate_connectivity of a
bmesh) have no counterpart here: no Blender session exists.
"""
from ..mesh import polygons_from_mesh, read_geometry_file

__all__ = ["read_geometry_file", "polygons_from_mesh"]
