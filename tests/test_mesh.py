"""STL geometry import (sparrowpy/utils/blender.py; tests/test_blender_import.py); .blend files in
test_blend.py.

The reference reads STL through Blender and checks, for a cube, that the
rough mesh keeps the fine mesh's vertices and has half as many faces.  The
same checks run here on cubes written as binary and ASCII STL (the
reference's cube.stl is a binary STL of the cube [-1, 1]^3 with 12
triangles), and the meshes feed DirectionalRadiosityFast.from_polygon: the
rough mesh as quadrilateral walls, the fine mesh as triangular walls cut
into triangular patches.
"""
import struct

import numpy as np
import numpy.testing as npt
import pytest

from sparrowpy_gb300 import DirectionalRadiosityFast
from sparrowpy_gb300.mesh import polygons_from_mesh, read_geometry_file
from sparrowpy_gb300.scenes import rotation_matrix_xyz


def cube_triangles(half=1.0, split_top=False):
    """Outward-wound triangles of the cube [-half, half]^3; the top face optionally as a 2 x 2 grid."""
    h = half
    quads = [  # counter-clockwise seen from outside
        [(-h, -h, h), (h, -h, h), (h, h, h), (-h, h, h)],
        [(-h, -h, -h), (-h, h, -h), (h, h, -h), (h, -h, -h)],
        [(-h, -h, -h), (h, -h, -h), (h, -h, h), (-h, -h, h)],
        [(-h, h, -h), (-h, h, h), (h, h, h), (h, h, -h)],
        [(-h, -h, -h), (-h, -h, h), (-h, h, h), (-h, h, -h)],
        [(h, -h, -h), (h, h, -h), (h, h, h), (h, -h, h)],
    ]
    tris = []
    for qi, q in enumerate(quads):
        q = np.asarray(q, float)
        if split_top and qi == 0:
            for a in range(2):
                for b in range(2):
                    x0, x1 = -h + a * h, -h + (a + 1) * h
                    y0, y1 = -h + b * h, -h + (b + 1) * h
                    sq = np.array([(x0, y0, h), (x1, y0, h), (x1, y1, h), (x0, y1, h)])
                    tris += [sq[[0, 1, 2]], sq[[0, 2, 3]]]
        else:
            tris += [q[[0, 1, 2]], q[[0, 2, 3]]]
    return np.array(tris)


def write_binary_stl(path, tris):
    with open(path, "wb") as f:
        f.write(b"written by the test".ljust(80, b"\0"))
        f.write(struct.pack("<I", len(tris)))
        for t in tris:
            f.write(struct.pack("<12fH", 0.0, 0.0, 0.0, *t.reshape(-1), 0))


def write_ascii_stl(path, tris):
    lines = ["solid cube"]
    for t in tris:
        lines += ["  facet normal 0 0 0", "    outer loop"]
        lines += [f"      vertex {v[0]:.9g} {v[1]:.9g} {v[2]:.9g}" for v in t]
        lines += ["    endloop", "  endfacet"]
    lines.append("endsolid cube")
    open(path, "w").write("\n".join(lines) + "\n")


@pytest.mark.parametrize("writer", [write_binary_stl, write_ascii_stl])
def test_mesh_simplification(tmp_path, writer):
    """tests/test_blender_import.py:8-15 for the STL cube."""
    path = tmp_path / "cube.stl"
    writer(path, cube_triangles())
    fine, rough = read_geometry_file(path)
    npt.assert_array_equal(fine["verts"], rough["verts"])
    assert len(fine["conn"]) == len(rough["conn"]) * 2
    assert fine["verts"].shape == (8, 3) and len(fine["conn"]) == 12
    assert all(len(p) == 4 for p in rough["conn"])


def test_rough_polygons_are_the_cube_faces(tmp_path):
    path = tmp_path / "cube.stl"
    write_binary_stl(path, cube_triangles(split_top=True))
    fine, rough = read_geometry_file(path)
    assert len(fine["conn"]) == 18 and fine["verts"].shape == (13, 3)
    assert len(rough["conn"]) == 6
    polys = polygons_from_mesh(rough)
    assert all(p.pts.shape == (4, 3) for p in polys)  # the split face's edge midpoints are left out
    npt.assert_allclose(sorted(p.area for p in polys), [4.0] * 6, rtol=1e-12)
    for p in polys:  # outward normals from the STL winding
        assert np.dot(p.normal, p.center) > 0
    inward = polygons_from_mesh(rough, flip=True)
    assert all(np.dot(p.normal, p.center) < 0 for p in inward)


@pytest.mark.parametrize("rotate", [False, True])
def test_stl_room_patches(tmp_path, rotate):
    """An STL room through from_polygon: 4 x 4 patches per 2 m face at 0.5 m, in any orientation."""
    tris = cube_triangles()
    if rotate:
        tris = tris @ rotation_matrix_xyz(0.3, 0.7, 1.1).T
    path = tmp_path / "room.stl"
    write_binary_stl(path, tris)  # float32 coordinates: a rotated face is planar to about 1e-7
    _, rough = read_geometry_file(path)
    r = DirectionalRadiosityFast.from_polygon(polygons_from_mesh(rough, flip=True), 0.5)
    assert r.n_patches == 6 * 16


def test_other_formats_and_bad_blend_files(tmp_path):
    with pytest.raises(NotImplementedError):
        read_geometry_file(tmp_path / "room.obj")
    bad = tmp_path / "room.blend"
    bad.write_bytes(b"not a blend file")
    with pytest.raises(ValueError):
        read_geometry_file(bad)


def _grid_triangles(cells, flip=()):
    """Triangles of unit squares (x, y) on z = 0, two per cell, counter-clockwise from +z; cells in `flip` have
    their first triangle wound the other way."""
    tris = []
    for k, (x, y) in enumerate(cells):
        sq = np.array([(x, y, 0.0), (x + 1, y, 0.0), (x + 1, y + 1, 0.0), (x, y + 1, 0.0)])
        t0 = sq[[0, 2, 1]] if k in flip else sq[[0, 1, 2]]
        tris += [t0, sq[[0, 2, 3]]]
    return np.array(tris)


def test_merged_face_with_a_hole_is_refused(tmp_path):
    """A 3 x 3 square with the middle cell missing: two boundary loops, which no single polygon holds."""
    ring = [(x, y) for x in range(3) for y in range(3) if (x, y) != (1, 1)]
    path = str(tmp_path / "ring.stl")
    write_binary_stl(path, _grid_triangles(ring))
    with pytest.raises(ValueError, match="holes are not supported"):
        read_geometry_file(path)
    # without the hole the same square merges into one quadrilateral
    path = str(tmp_path / "square.stl")
    write_binary_stl(path, _grid_triangles([(x, y) for x in range(3) for y in range(3)]))
    _, rough = read_geometry_file(path)
    assert len(rough["conn"]) == 1 and len(rough["conn"][0]) == 4


def test_inconsistent_winding_stays_a_face_of_its_own(tmp_path):
    """A triangle wound against its neighbours has the opposite normal, so it is not merged with them: the
    rest of the square merges into one polygon around it, and the triangle stays a face of its own."""
    path = str(tmp_path / "flipped.stl")
    write_binary_stl(path, _grid_triangles([(x, y) for x in range(2) for y in range(2)], flip=(3,)))
    _, rough = read_geometry_file(path)
    sizes = sorted(len(c) for c in rough["conn"])
    assert sizes[0] == 3 and len(sizes) == 2


def test_stl_fine_mesh_room_patches(tmp_path):
    """The fine mesh (the file's own triangles) as walls: triangular patches tiling each triangle."""
    path = tmp_path / "room.stl"
    write_binary_stl(path, cube_triangles())
    fine, _ = read_geometry_file(path)
    walls = polygons_from_mesh(fine, flip=True)
    assert all(p.pts.shape == (3, 3) for p in walls)
    r = DirectionalRadiosityFast.from_polygon(walls, 0.5)
    assert r._patches_points.shape[1:] == (3, 3)
    assert r.n_patches == 12 * 25  # each half-face triangle: longest side 2.83 m, cut 5 x 5 at 0.5 m
    areas = np.array([0.5 * np.linalg.norm(np.cross(p[1] - p[0], p[2] - p[0])) for p in r._patches_points])
    npt.assert_allclose(areas.sum(), 24.0, rtol=1e-6)


@pytest.mark.gpu
def test_stl_fine_mesh_room_matches_oracle(tmp_path):
    """The STL cube's fine mesh (12 triangles) as a room of triangular patches, FP64 on the GPU against the
    oracle."""
    from oracle import oracle as orc
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    path = tmp_path / "room.stl"
    write_binary_stl(path, cube_triangles())
    fine, _ = read_geometry_file(path)
    r = DirectionalRadiosityFast.from_polygon(polygons_from_mesh(fine, flip=True), 1.0, precision="fp64")
    f = np.array([1000.0])
    dirs = hemisphere_directions(8)
    brdf = create_from_scattering(dirs, dirs, FrequencyData([0.5], f), FrequencyData([0.2], f))
    r.set_wall_brdf(np.arange(12), brdf, dirs, dirs)
    r.set_air_attenuation(FrequencyData([0.0], f))
    src, rcv = np.array([0.2, -0.3, 0.1]), np.array([[-0.4, 0.5, -0.2]])
    c, dt, dur, k = 343.0, 1e-3, 0.05, 5
    r.bake_geometry()
    r.init_source_energy(Coordinates(*src))
    r.calculate_energy_exchange(c, dt, dur, k)
    mono = r.collect_energy_receiver_mono(Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])).time
    ref = orc.solve(scene_from_radiosity(r), src, rcv, c, dt, dur, k)
    np.testing.assert_array_equal(r._visibility_matrix, ref["bake"]["vis"])
    assert np.sum(ref["mono"]) > 0
    assert np.linalg.norm(mono - ref["mono"]) / np.linalg.norm(ref["mono"]) < 1e-10
