"""Triangles and other convex polygons as patches.

The reference's universal form factor, its Stokes and Nusselt integrals and
its point factor accept polygons of any vertex count (universal.py:54-96,
integration.py:38-344); its own tests use quadrilaterals only.  Golden
values of the reference on seeded triangles, pentagons and hexagons (facing,
hinged on a shared side, sharing a vertex, randomly placed, triangles
against quadrilaterals) and point factors of triangles and pentagons are in
tests/golden/polygons.npz (tests/golden/make_polygon_golden.py):

* the oracle against them, relative 1e-12 (CPU);
* sp_form_factors on patches of 3, 5 and 6 vertices against them: FP64
  results within 1e-10 (pentagons and hexagons always FP64, one warp per
  pair), FP32 Stokes results of triangles within 1e-5;
* the point factors of sp_source_energy and sp_receiver_factors against
  them, relative 1e-12.

The whole pipeline on triangular patches (the reference-run `tri` scene) is
checked in test_oracle_golden.py and test_gpu_parity.py.
"""
import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as orc


@pytest.fixture(scope="module")
def golden():
    return load_golden("polygons")


def _poly_area(p):
    return sum(0.5 * np.linalg.norm(np.cross(p[t + 1] - p[0], p[t + 2] - p[0])) for t in range(len(p) - 2))


def test_oracle_polygon_form_factors(golden):
    g = golden
    for k in range(g["value"].size):
        a, b = g["pi"][k, :g["nvi"][k]], g["pj"][k, :g["nvj"][k]]
        if g["nusselt"][k]:
            v = orc.nusselt(a, b, g["ni"][k], g["nj"][k])
        else:
            v = orc.stokes(a, b, g["area_i"][k])
        assert abs(v - g["value"][k]) <= 1e-12 * abs(g["value"][k]), (str(g["kinds"][k]), k)


def test_oracle_polygon_point_factors(golden):
    g = golden
    for k in range(g["pt_value"].size):
        mode = "source" if g["pt_mode"][k] == 0 else "receiver"
        v = orc.pt_solution(g["pt_point"][k], g["pt_poly"][k, :g["pt_nv"][k]], mode)
        assert abs(v - g["pt_value"][k]) <= 1e-12 * abs(g["pt_value"][k]), k


def test_oracle_universal_same_vertex_count(golden):
    """orc_form_factors (the pair list entry point) decides Stokes or Nusselt as universal.py:54-96 does."""
    g = golden
    for nv in (3, 5, 6):
        sel = np.flatnonzero((g["nvi"] == nv) & (g["nvj"] == nv))
        pts = np.concatenate([np.stack([g["pi"][k, :nv], g["pj"][k, :nv]]) for k in sel])
        normals = np.concatenate([np.stack([g["ni"][k], g["nj"][k]]) for k in sel])
        areas = np.array([_poly_area(p) for p in pts])
        pairs = np.stack([2 * np.arange(sel.size), 2 * np.arange(sel.size) + 1], axis=1)
        ff = orc.form_factors(pts, normals, areas, pairs)
        np.testing.assert_allclose(ff, g["value"][sel], rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_gpu_polygon_form_factors(golden, precision):
    import torch
    from sparrowpy_gb300 import _native as nat
    g = golden
    for nv in (3, 5, 6):
        sel = np.flatnonzero((g["nvi"] == nv) & (g["nvj"] == nv))
        pts = np.concatenate([np.stack([g["pi"][k, :nv], g["pj"][k, :nv]]) for k in sel])
        normals = np.concatenate([np.stack([g["ni"][k], g["nj"][k]]) for k in sel])
        areas = np.array([_poly_area(p) for p in pts])
        pairs = np.stack([2 * np.arange(sel.size), 2 * np.arange(sel.size) + 1], axis=1).astype(np.int32)
        dev = lambda x, t: torch.as_tensor(np.ascontiguousarray(x), dtype=t, device="cuda")
        p, nr, ar, pr = (dev(pts, torch.float64), dev(normals, torch.float64), dev(areas, torch.float64),
                         dev(pairs, torch.int32))
        m = sel.size
        ff = torch.zeros((m,), dtype=torch.float64, device="cuda")
        method = torch.zeros((m,), dtype=torch.uint8, device="cuda")
        wsz = nat.size("sp_form_factors_workspace", pts.shape[0], m)
        ws = torch.empty((max(wsz, 1),), dtype=torch.uint8, device="cuda")
        nat.call("sp_form_factors", nat.SP_F32 if precision == "fp32" else nat.SP_F64, pts.shape[0], nv, m,
                 pr.data_ptr(), p.data_ptr(), nr.data_ptr(), ar.data_ptr(), ff.data_ptr(), method.data_ptr(),
                 ws.data_ptr(), wsz, torch.cuda.current_stream().cuda_stream)
        got, meth = ff.cpu().numpy(), method.cpu().numpy()
        rel = np.abs(got - g["value"][sel]) / np.abs(g["value"][sel])
        # Nusselt for the pairs sharing a vertex; Stokes for the others: FP32 (method 0, triangles in FP32)
        # within 1e-5, FP64 (method 1) within 1e-10
        np.testing.assert_array_equal(meth == 2, g["nusselt"][sel])
        assert rel[meth != 0].max(initial=0) < 1e-10, nv
        assert rel[meth == 0].max(initial=0) < 1e-5, nv
        if precision == "fp64" or nv > 3:
            assert (meth != 0).all()


@pytest.mark.gpu
def test_gpu_polygon_point_factors(golden):
    import torch
    from sparrowpy_gb300 import _native as nat
    g = golden
    dev = lambda x, t: torch.as_tensor(np.ascontiguousarray(x), dtype=t, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    ones = dict(vis=dev(np.ones(1), torch.uint8), wall=dev(np.zeros(1), torch.int32),
                slot=dev(np.zeros(1), torch.int32), dirs=dev(np.array([[[0, 0, 1.0]]]), torch.float64),
                brdf=dev(np.ones((1, 1, 1, 1)), torch.float64), att=dev(np.zeros(1), torch.float64))
    for k in range(g["pt_value"].size):
        nv = int(g["pt_nv"][k])
        poly = g["pt_poly"][k, :nv]
        p, c, x = dev(poly, torch.float64), dev(poly.mean(axis=0), torch.float64), dev(g["pt_point"][k],
                                                                                       torch.float64)
        if g["pt_mode"][k] == 0:
            e0 = torch.empty((1, 1), dtype=torch.float64, device="cuda")
            d0 = torch.empty((1,), dtype=torch.float64, device="cuda")
            e0dir = torch.empty((1, 1, 1), dtype=torch.float64, device="cuda")
            nat.call("sp_source_energy", x.data_ptr(), 1, c.data_ptr(), p.data_ptr(), nv, ones["vis"].data_ptr(),
                     1, ones["att"].data_ptr(), ones["wall"].data_ptr(), ones["slot"].data_ptr(), 1,
                     ones["dirs"].data_ptr(), 1, ones["brdf"].data_ptr(), e0.data_ptr(), d0.data_ptr(),
                     e0dir.data_ptr(), st)
            got = float(e0.cpu()[0, 0])
        else:
            rfac = torch.empty((1,), dtype=torch.float64, device="cuda")
            ridx = torch.empty((1,), dtype=torch.int32, device="cuda")
            dist = torch.empty((1,), dtype=torch.float64, device="cuda")
            nat.call("sp_receiver_factors", x.data_ptr(), 1, c.data_ptr(), p.data_ptr(), nv, ones["vis"].data_ptr(),
                     ones["wall"].data_ptr(), 1, ones["dirs"].data_ptr(), rfac.data_ptr(), ridx.data_ptr(),
                     dist.data_ptr(), st)
            got = float(rfac.cpu()[0])
        assert abs(got - g["pt_value"][k]) <= 1e-12 * abs(g["pt_value"][k]), k


def test_bake_rejects_unsupported_vertex_counts():
    from sparrowpy_gb300 import DirectionalRadiosityFast
    walls = np.array([[[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]], dtype=float)
    nine = np.stack([np.array([np.cos(a), np.sin(a), 0.0]) for a in np.linspace(0, 2 * np.pi, 9, endpoint=False)])
    r = DirectionalRadiosityFast(walls, np.array([[0, 0, 1.0]]), np.array([[1.0, 0, 0]]), nine[None], 1, [0])
    with pytest.raises(NotImplementedError):
        r.bake_geometry()


def test_walls_of_mixed_vertex_counts_are_refused():
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.geometry import Polygon
    quad = Polygon([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], [1, 0, 0], [0, 0, 1])
    tri = Polygon([[0, 0, 1], [0, 1, 1], [1, 0, 1]], [0, 1, 0], [0, 0, -1])
    with pytest.raises(ValueError, match="vertex counts"):
        DirectionalRadiosityFast.from_polygon([quad, tri], 0.5)
