"""Room geometry from STL and .blend files (sparrowpy/utils/blender.py:22-142, without Blender).

The reference reads .blend and .stl files through Blender's Python modules
(bpy, bmesh) and returns two meshes: the file's own faces ("fine") and the
faces merged across edges whose normals differ by less than an angular
tolerance ("rough", bmesh.ops.dissolve_limit).  Blender is not available
here, so this module reads the files directly:

* fine: an STL file's triangles with identical vertices welded, or the
  mesh of a .blend file's object "Geometry" as stored (blend.py), its
  vertices and faces in the file's order;
* rough: edge-connected faces whose normals differ by less than
  angular_tolerance merged into polygons, each traced as its boundary loop.
  A loop vertex where the boundary runs straight on (turn below the
  tolerance) is left out of that polygon.  `verts` keeps every vertex, so
  the two meshes share it, as the reference's test expects for a cube.

polygons_from_mesh turns a mesh into Polygon objects (vertices projected
onto each polygon's plane) for DirectionalRadiosityFast.from_polygon, which
patches quadrilateral walls in any orientation and cuts the walls of other
vertex counts (the fine mesh's triangles) into triangular patches.
"""
import os
import struct

import numpy as np

from .geometry import Polygon


def _read_stl(path):
    """Triangles (n, 3, 3) of a binary or ASCII STL file."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) >= 84:
        n = struct.unpack("<I", data[80:84])[0]
        if len(data) == 84 + 50 * n:  # binary
            rec = np.frombuffer(data, dtype=np.dtype([("n", "<f4", 3), ("v", "<f4", (3, 3)), ("a", "<u2")]),
                                count=n, offset=84)
            return rec["v"].astype(np.float64)
    text = data.decode("ascii", errors="strict")
    if not text.lstrip().lower().startswith("solid"):
        raise ValueError(f"{path}: not an STL file")
    verts = [list(map(float, line.split()[1:4])) for line in text.splitlines() if line.strip().startswith("vertex")]
    if len(verts) % 3:
        raise ValueError(f"{path}: the facets do not have three vertices each")
    return np.asarray(verts, dtype=np.float64).reshape(-1, 3, 3)


def _weld(tris):
    """Unique vertices (first-seen order) and the triangles as index triples."""
    flat = tris.reshape(-1, 3)
    _, first, inverse = np.unique(flat, axis=0, return_index=True, return_inverse=True)
    order = np.argsort(first)                     # unique vertices in order of first appearance
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    return flat[first[order]], rank[inverse.reshape(-1)].reshape(-1, 3)


def _normal(pts):
    """Unit normal of a polygon (Newell's method)."""
    n = np.zeros(3)
    for k in range(len(pts)):
        a, b = pts[k], pts[(k + 1) % len(pts)]
        n += np.array([(a[1] - b[1]) * (a[2] + b[2]), (a[2] - b[2]) * (a[0] + b[0]), (a[0] - b[0]) * (a[1] + b[1])])
    nn = np.linalg.norm(n)
    return n / nn if nn > 0 else n


def _merge_coplanar(verts, faces, angular_tolerance):
    """Polygons (vertex index loops) of edge-connected faces whose normals agree within the tolerance."""
    cos_tol = np.cos(np.deg2rad(angular_tolerance))
    normals = np.array([_normal(verts[f]) for f in faces])
    parent = list(range(len(faces)))

    def find(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    edge_faces = {}
    for fi, f in enumerate(faces):
        for k in range(len(f)):
            e = (min(f[k], f[(k + 1) % len(f)]), max(f[k], f[(k + 1) % len(f)]))
            edge_faces.setdefault(e, []).append(fi)
    for fs in edge_faces.values():
        if len(fs) == 2 and normals[fs[0]] @ normals[fs[1]] >= cos_tol:
            a, b = find(fs[0]), find(fs[1])
            if a != b:
                parent[max(a, b)] = min(a, b)
    regions = {}
    for fi in range(len(faces)):
        regions.setdefault(find(fi), []).append(fi)
    polys = []
    for root in sorted(regions):
        members = regions[root]
        # boundary edges: edges used by one face of the region (counted without
        # direction, so that faces wound inconsistently still share their
        # inner edges), each in its face's direction
        uses = {}
        for fi in members:
            f = faces[fi]
            for k in range(len(f)):
                a, b = int(f[k]), int(f[(k + 1) % len(f)])
                uses.setdefault((min(a, b), max(a, b)), []).append((a, b))
        nxt = {}
        for used in uses.values():
            if len(used) != 1:
                continue
            a, b = used[0]
            if a in nxt:
                raise ValueError("a merged region's boundary has a vertex with two outgoing edges "
                                 "(faces wound inconsistently, or regions touching at a vertex)")
            nxt[a] = b
        if not nxt:
            continue
        start = min(nxt)
        loop, v = [start], nxt.get(start)
        while v is not None and v != start and len(loop) <= len(nxt):
            loop.append(v)
            v = nxt.get(v)
        if v != start or len(loop) != len(nxt):
            # an open chain, or boundary edges left over after one closed loop:
            # a hole (a second loop) or an inconsistently wound face
            raise ValueError("a merged region's boundary is not one simple loop (holes are not supported)")
        # leave out loop vertices where the boundary runs straight on
        keep = []
        for k, vi in enumerate(loop):
            a, b, c = verts[loop[k - 1]], verts[vi], verts[loop[(k + 1) % len(loop)]]
            u, w = b - a, c - b
            cosang = (u @ w) / (np.linalg.norm(u) * np.linalg.norm(w))
            if cosang < cos_tol:
                keep.append(vi)
        polys.append(keep)
    return polys


def read_geometry_file(path, angular_tolerance=3.):
    """Fine and rough meshes of a geometry file (sparrowpy/utils/blender.py:22-97).

    Returns two dicts {"verts": (n, 3) array, "conn": list of vertex index
    lists}: the file's faces and the polygons of faces merged within
    angular_tolerance degrees.
    """
    ext = os.path.splitext(str(path))[-1].lower()
    if ext == ".blend":
        from .blend import read_mesh
        verts, faces = read_mesh(path)
        fine = {"verts": verts, "conn": [list(map(int, f)) for f in faces]}
        rough = {"verts": verts,
                 "conn": [list(map(int, p)) for p in _merge_coplanar(verts, faces, angular_tolerance)]}
        return fine, rough
    if ext != ".stl":
        raise NotImplementedError("Only .stl and .blend files are supported.")
    verts, faces = _weld(_read_stl(path))
    fine = {"verts": verts, "conn": [list(map(int, f)) for f in faces]}
    rough = {"verts": verts, "conn": [list(map(int, p)) for p in _merge_coplanar(verts, faces, angular_tolerance)]}
    return fine, rough


def polygons_from_mesh(mesh, flip=False):
    """Polygon objects of a mesh: normal from the vertex order (flip=True reverses it), up vector along the
    first edge.

    STL stores float32 coordinates, so a face that is not aligned with the
    axes is planar only to about 1e-7; Polygon (as the reference's) wants
    1e-10.  Each polygon's vertices are therefore projected onto its plane
    (through their mean, along the Newell normal) first.
    """
    out = []
    for conn in mesh["conn"]:
        idx = list(conn)[::-1] if flip else list(conn)
        pts = np.asarray(mesh["verts"], dtype=float)[idx]
        n = _normal(pts)
        c = pts.mean(axis=0)
        pts = pts - np.outer((pts - c) @ n, n)
        up = pts[1] - pts[0]
        out.append(Polygon(pts, up / np.linalg.norm(up), n))
    return out
