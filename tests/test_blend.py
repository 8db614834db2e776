"""Room geometry from .blend files without Blender (blend.py, mesh.py).

Restates the reference's tests that need Blender (skipped there without
bpy): tests/test_blender_import.py:9-16 (the fine and rough meshes of
cube.blend share their vertices, the fine mesh has twice the faces) and
tests/test_visibility.py:75-139 (the patch-to-patch visibility of the fine
meshes of cube_simple.blend, cube.blend and cube_blocked.blend against
known solutions: every pair; pairs whose ray leaves patch i on its front;
the test file's list of visible pairs).  The meshes and the list come from
tests/golden/blend.npz (make_blend_golden.py); with SPARROWPY_SRC set, the
files themselves are read again and compared.  Visibility: the oracle on
the CPU, sp_patch_visibility on the GPU, both with the fine mesh's patches
as blockers.
"""
import hashlib
import os

import numpy as np
import numpy.testing as npt
import pytest

from conftest import load_golden
from sparrowpy_gb300 import mesh

SRC = os.environ.get("SPARROWPY_SRC")
MODELS = ("cube_simple", "cube", "cube_blocked")


@pytest.fixture(scope="module")
def gold():
    return load_golden("blend")


def fine_mesh(g, name):
    faces = [[int(i) for i in row if i >= 0] for row in g[f"{name}_faces"]]
    return np.asarray(g[f"{name}_verts"], float), faces


def patches_of(verts, faces):
    pts = np.stack([verts[f] for f in faces])
    ctr = pts.sum(axis=1) / pts.shape[1]
    nrm = np.cross(pts[:, 1] - pts[:, 0], pts[:, 2] - pts[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    return pts, ctr, nrm


def solution(g, name, ctr, nrm):
    n = ctr.shape[0]
    sol = np.zeros((n, n), dtype=bool)
    if name == "cube_simple":
        sol[np.triu_indices(n, 1)] = True
    elif name == "cube":
        for i in range(n):
            for j in range(i + 1, n):
                ray = (ctr[j] - ctr[i]) / np.linalg.norm(ctr[j] - ctr[i])
                sol[i, j] = nrm[i] @ ray > 1e-6
    else:
        for i, j in g["cube_blocked_visible"]:
            sol[i, j] = True
    return sol


def test_cube_fine_and_rough_meshes(gold):
    """tests/test_blender_import.py:9-16 on the stored cube.blend mesh: the rough mesh (faces merged within 3
    degrees) keeps the fine mesh's vertices and has half its faces."""
    verts, faces = fine_mesh(gold, "cube")
    rough = mesh._merge_coplanar(verts, faces, 3.0)
    assert len(faces) == 2 * len(rough)
    assert set(i for p in rough for i in p) == set(i for f in faces for i in f)
    assert all(len(p) == 4 for p in rough)


@pytest.mark.parametrize("name", MODELS)
def test_oracle_visibility_of_blend_meshes(gold, name):
    from oracle import oracle as orc
    verts, faces = fine_mesh(gold, name)
    pts, ctr, nrm = patches_of(verts, faces)
    npt.assert_array_equal(orc.patch_visibility(ctr, nrm, pts), solution(gold, name, ctr, nrm))


@pytest.mark.gpu
@pytest.mark.parametrize("name", MODELS)
def test_gpu_visibility_of_blend_meshes(gold, name):
    import torch
    from sparrowpy_gb300 import _native as nat
    verts, faces = fine_mesh(gold, name)
    pts, ctr, nrm = patches_of(verts, faces)
    n, nv = pts.shape[0], pts.shape[1]
    dev = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")
    vis = torch.empty((n, n), dtype=torch.uint8, device="cuda")
    wsz = nat.size("sp_patch_visibility_workspace", n)
    ws = torch.empty((max(wsz, 1),), dtype=torch.uint8, device="cuda")
    c, nr, p = dev(ctr), dev(nrm), dev(pts)
    nat.call("sp_patch_visibility", n, nv, c.data_ptr(), nr.data_ptr(), p.data_ptr(), vis.data_ptr(), ws.data_ptr(),
             wsz, torch.cuda.current_stream().cuda_stream)
    npt.assert_array_equal(vis.cpu().numpy().astype(bool), solution(gold, name, ctr, nrm))


@pytest.mark.skipif(not SRC, reason="the reference's .blend files are read when SPARROWPY_SRC is set")
def test_blend_reader_against_stored_meshes(gold):
    for name in MODELS:
        path = os.path.join(SRC, "tests", "test_data", name + ".blend")
        with open(path, "rb") as fh:
            assert hashlib.sha256(fh.read()).hexdigest() == str(gold[f"{name}_sha256"])
        fine, rough = mesh.read_geometry_file(path)
        verts, faces = fine_mesh(gold, name)
        npt.assert_array_equal(fine["verts"], verts)
        assert fine["conn"] == faces
    fine, rough = mesh.read_geometry_file(os.path.join(SRC, "tests", "test_data", "cube.blend"))
    npt.assert_array_equal(fine["verts"], rough["verts"])
    assert len(fine["conn"]) == len(rough["conn"]) * 2


@pytest.mark.gpu
def test_gpu_blocked_cube_room_matches_oracle(gold):
    """cube_blocked.blend's fine mesh (16 triangles: a box with a wedge pushed in from one side) as a room of
    triangular patches, source and receiver on either side of the wedge: FP64 on the GPU against the
    oracle (visibility exact, receiver histogram 1e-10)."""
    from oracle import oracle as orc
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    from sparrowpy_gb300.radiosity import DirectionalRadiosityFast
    verts, faces = fine_mesh(gold, "cube_blocked")
    walls = mesh.polygons_from_mesh({"verts": verts, "conn": faces})  # its faces are wound towards the room
    r = DirectionalRadiosityFast.from_polygon(walls, 1.0, precision="fp64")
    f = np.array([1000.0])
    dirs = hemisphere_directions(8)
    brdf = create_from_scattering(dirs, dirs, FrequencyData([0.5], f), FrequencyData([0.2], f))
    r.set_wall_brdf(np.arange(len(walls)), brdf, dirs, dirs)
    r.set_air_attenuation(FrequencyData([0.0], f))
    src, rcv = np.array([0.5, 0.9, 1.0]), np.array([[0.5, -0.9, 1.0]])
    c, dt, dur, k = 343.0, 1e-3, 0.05, 5
    r.bake_geometry()
    r.init_source_energy(Coordinates(*src))
    r.calculate_energy_exchange(c, dt, dur, k)
    mono = r.collect_energy_receiver_mono(Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])).time
    ref = orc.solve(scene_from_radiosity(r), src, rcv, c, dt, dur, k)
    np.testing.assert_array_equal(r._visibility_matrix, ref["bake"]["vis"])
    assert np.sum(ref["mono"]) > 0
    assert np.linalg.norm(mono - ref["mono"]) / np.linalg.norm(ref["mono"]) < 1e-10
