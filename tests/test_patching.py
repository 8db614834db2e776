"""Wall patching (sparrowpy/geometry.py:290-410) and its extensions: walls in any orientation, triangles.

Axis-aligned walls keep the reference's arithmetic bit for bit.  Walls the
reference cannot patch (no coordinate axis spans less than the patch size)
are split along their own edges; a rotated room then gives the same patches
as the rotated patches of the axis-aligned room, and its solve on the GPU
matches the oracle on the same patches.  Walls of other vertex counts (a
tetrahedron room) are cut into triangular patches that tile them, and that
room's GPU solve matches the oracle too.
"""
import numpy as np
import numpy.testing as npt
import pytest

from sparrowpy_gb300 import geometry as geo
from sparrowpy_gb300.geometry import Polygon, shoebox_room_stub
from sparrowpy_gb300.scenes import rotation_matrix_xyz

ROT = rotation_matrix_xyz(0.3, 0.7, 1.1)
SHIFT = np.array([0.37, -1.21, 0.53])


def rotated(polys):
    return [Polygon(np.asarray(p.pts) @ ROT.T + SHIFT, np.asarray(p.up_vector) @ ROT.T, np.asarray(p.normal) @ ROT.T)
            for p in polys]


def test_axis_aligned_walls_keep_reference_patches():
    walls = shoebox_room_stub(3, 2, 2)
    pts = np.array([w.pts for w in walls], float)
    nrm = np.array([w.normal for w in walls], float)
    got, _, n, ids = geo.process_patches(pts, nrm, 0.5)
    ref = np.concatenate([geo.create_patches(w, 0.5) for w in pts])
    npt.assert_array_equal(got, ref)
    assert n == 2 * (6 * 4 + 6 * 4 + 4 * 4)
    npt.assert_array_equal(np.bincount(ids), [24, 24, 24, 24, 16, 16])


def test_rotated_wall_patches_tile_the_wall():
    wall = np.array([[0, 0, 0], [3, 0, 0], [3, 0, 2], [0, 0, 2]], float) @ ROT.T + SHIFT
    assert not geo.axis_patchable(wall, 0.5)
    with pytest.raises(ValueError):
        geo.create_patches(wall, 0.5)  # the reference's patching does not apply
    p = geo.create_patches_general(wall, 0.5)
    assert p.shape == (6 * 4, 4, 3)
    area = geo.calculate_area(p)
    npt.assert_allclose(area, 0.25, rtol=1e-12)
    npt.assert_allclose(area.sum(), 6.0, rtol=1e-12)
    n = np.cross(wall[1] - wall[0], wall[3] - wall[0])
    n /= np.linalg.norm(n)
    npt.assert_allclose((p.reshape(-1, 3) - wall[0]) @ n, 0.0, atol=1e-12)
    # each patch keeps the wall's orientation
    pn = np.cross(p[:, 1] - p[:, 0], p[:, 3] - p[:, 0])
    assert np.all(pn @ n > 0)


def test_rotated_room_patches_are_the_rotated_patches():
    walls = shoebox_room_stub(3, 2, 2)
    ref, _, _, ref_ids = geo.process_patches(np.array([w.pts for w in walls]), np.array([w.normal for w in walls]), 0.5)
    rw = rotated(walls)
    got, _, _, ids = geo.process_patches(np.array([w.pts for w in rw]), np.array([w.normal for w in rw]), 0.5)
    npt.assert_array_equal(np.bincount(ids), np.bincount(ref_ids))
    want = geo.calculate_center(ref) @ ROT.T + SHIFT
    have = geo.calculate_center(got)
    for w in range(len(walls)):
        a = want[ref_ids == w]
        b = have[ids == w]
        d = np.linalg.norm(a[:, None, :] - b[None, :, :], axis=-1)
        assert np.all(d.min(axis=1) < 1e-12)


@pytest.mark.parametrize("pts", [
    [[0, 0, 0], [1, 0, 0.3], [1, 1, 0], [0, 1, 0.1]],          # not planar
    [[0, 0, 0], [2, 0, 0], [0.5, 0.5, 0], [0, 2, 0]],          # not convex
    [[0, 0, 0], [1, 0, 0], [2, 0, 0], [3, 0, 0]],              # degenerate
])
def test_general_patching_rejects_bad_walls(pts):
    pts = np.asarray(pts, float) @ ROT.T
    with pytest.raises(ValueError):
        geo.create_patches_general(pts, 0.5)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_rotated_room_matches_oracle(precision):
    """A room in a general orientation, patched by from_polygon, through the GPU path against the oracle."""
    from oracle import oracle as orc
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    f = np.array([500.0, 1000.0])
    dirs = hemisphere_directions(8)
    src = np.array([0.6, 0.5, 1.3]) @ ROT.T + SHIFT
    rcv = np.array([[2.4, 1.5, 0.9], [0.5, 1.6, 1.6]]) @ ROT.T + SHIFT
    walls = rotated(shoebox_room_stub(3, 2, 2))
    r = DirectionalRadiosityFast.from_polygon(walls, 0.5, precision=precision)
    assert r.n_patches == 2 * (24 + 24 + 16)
    brdf = create_from_scattering(dirs, dirs, FrequencyData([0.3, 0.6], f), FrequencyData([0.1, 0.2], f))
    r.set_wall_brdf(np.arange(len(walls)), brdf, dirs, dirs)
    r.set_air_attenuation(FrequencyData([0.001, 0.002], f))
    c, dt, dur, k = 343.0, 1e-3, 0.1, 8
    r.bake_geometry()
    r.init_source_energy(Coordinates(*src))
    r.calculate_energy_exchange(c, dt, dur, k)
    mono = r.collect_energy_receiver_mono(Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])).time
    ref = orc.solve(scene_from_radiosity(r), src, rcv, c, dt, dur, k)
    np.testing.assert_array_equal(r._visibility_matrix, ref["bake"]["vis"])
    assert np.sum(ref["mono"]) > 0
    tol = 1e-10 if precision == "fp64" else 1e-4
    rel = np.linalg.norm(mono - ref["mono"]) / np.linalg.norm(ref["mono"])
    assert rel < tol


# ------------------------------------------------------------- triangles
def tetrahedron(scale=2.5):
    """A closed tetrahedron room, each wall wound so that its normal points inside."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0.3, 0.9, 0], [0.35, 0.3, 0.85]], float) * scale @ ROT.T + SHIFT
    inner = v.mean(axis=0)
    walls = []
    for f in ((0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3)):
        p = v[list(f)]
        n = np.cross(p[1] - p[0], p[2] - p[0])
        if n @ (inner - p[0]) < 0:
            p, n = p[::-1], -n
        up = p[1] - p[0]
        walls.append(Polygon(p, up / np.linalg.norm(up), n / np.linalg.norm(n)))
    return walls, v, inner


def test_triangle_patches_tile_the_wall():
    walls, _, _ = tetrahedron()
    for w in walls:
        p = geo.create_patches_triangles(w.pts, 0.5)
        area = geo.calculate_area(p)
        npt.assert_allclose(area.sum(), geo.calculate_area(np.asarray(w.pts)[None])[0], rtol=1e-12)
        npt.assert_allclose(area, area[0], rtol=1e-9)  # similar triangles of one wall
        npt.assert_allclose((p.reshape(-1, 3) - w.pts[0]) @ w.normal, 0.0, atol=1e-12)
        pn = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
        assert np.all(pn @ w.normal > 0)  # the wall's orientation
    # a convex pentagon: the fan of 3 triangles, each cut into n x n
    pent = np.stack([[np.cos(a), np.sin(a), 0.0] for a in np.linspace(0, 2 * np.pi, 5, endpoint=False)])
    p = geo.create_patches_triangles(pent, 0.5)
    npt.assert_allclose(geo.calculate_area(p).sum(), 2.5 * np.sin(2 * np.pi / 5), rtol=1e-12)
    pts, normals, n, ids = geo.process_patches(np.array([w.pts for w in walls]), np.array([w.normal for w in walls]),
                                               0.5)
    assert pts.shape[1:] == (3, 3) and n == pts.shape[0] and np.bincount(ids).min() > 1


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_triangle_room_matches_oracle(precision):
    """A tetrahedron room in a general orientation, triangular walls cut into triangular patches by
    from_polygon, through the GPU path against the oracle (form factors: FP32 Stokes pairs within 1e-5, the
    FP64 ones within 1e-10)."""
    from oracle import oracle as orc
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    f = np.array([500.0, 1000.0])
    dirs = hemisphere_directions(8)
    walls, v, inner = tetrahedron()
    src = inner + 0.1 * (v[1] - inner)
    rcv = np.stack([inner + 0.2 * (v[2] - inner), inner + 0.3 * (v[3] - inner)])
    r = DirectionalRadiosityFast.from_polygon(walls, 0.5, precision=precision)
    assert r._patches_points.shape[1] == 3 and r.n_patches > 50
    brdf = create_from_scattering(dirs, dirs, FrequencyData([0.3, 0.6], f), FrequencyData([0.1, 0.2], f))
    r.set_wall_brdf(np.arange(len(walls)), brdf, dirs, dirs)
    r.set_air_attenuation(FrequencyData([0.001, 0.002], f))
    c, dt, dur, k = 343.0, 1e-3, 0.1, 8
    r.bake_geometry()
    r.init_source_energy(Coordinates(*src))
    r.calculate_energy_exchange(c, dt, dur, k)
    mono = r.collect_energy_receiver_mono(Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])).time
    ref = orc.solve(scene_from_radiosity(r), src, rcv, c, dt, dur, k)
    np.testing.assert_array_equal(r._visibility_matrix, ref["bake"]["vis"])
    ff = r._form_factors[ref["bake"]["pairs"][:, 0], ref["bake"]["pairs"][:, 1]]
    method = r._bake["ff_method"].cpu().numpy()[: ff.size]
    rel = np.abs(ff - ref["bake"]["ff"]) / np.abs(ref["bake"]["ff"])
    assert rel[method != 0].max(initial=0) < 1e-10  # FP64 Stokes and Nusselt pairs
    assert rel[method == 0].max(initial=0) < 1e-5   # FP32 Stokes pairs (precision "fp32")
    assert precision == "fp32" or (method != 0).all()
    assert np.sum(ref["mono"]) > 0
    tol = 1e-10 if precision == "fp64" else 1e-4
    rel = np.linalg.norm(mono - ref["mono"]) / np.linalg.norm(ref["mono"])
    assert rel < tol
