"""Known-answer cases of the reference's own test suite, restated without pyfar.

Each test names the sparrowpy test it follows and keeps its tolerance:

* form factors of rectangle pairs against analytic view factors
  (tests/test_universal_formfactor.py:11-137): parallel facing < 1.5 %,
  perpendicular with a common edge < 2 %, perpendicular with a common
  vertex < 5 %.  Pinned on the oracle (CPU) and on the GPU in both precisions;
* ff_tilde row sums in closed shoeboxes (:140-157), within 1e-2;
* reciprocity of F' for different areas (:160-206);
* cube visibility pattern (tests/test_DRadiosityFast.py:19-29) and the
  outgoing-direction map of two perpendicular walls (:46-107);
* the infinite diffuse plane of Svensson and Savioja (2024)
  (tests/test_DRadiosityFast_infinite_diffuse_plane.py:96-155);
* source-receiver reciprocity of the room response
  (tests/test_multisource.py:51-137) and of the point factors (:140-213);
* one call with many receivers equal to single-receiver calls (:10-48);
* source and receiver visibility (tests/test_visibility.py:209-247).

The analytic view factors are the published closed forms: directly opposed
parallel rectangles (Howell's catalogue, C-11) and perpendicular rectangles
in general position by the corner-function sum of Ehlert and Smith (1993),
which contains the common-edge (C-14) and common-vertex cases.
"""
import itertools

import numpy as np
import pytest

# ------------------------------------------------------------ analytic view factors


def ff_parallel(a, b, c):
    """Directly opposed parallel a x b rectangles at distance c."""
    x, y = a / c, b / c
    return 2 / (np.pi * x * y) * (
        0.5 * np.log((1 + x * x) * (1 + y * y) / (1 + x * x + y * y))
        + x * np.sqrt(1 + y * y) * np.arctan(x / np.sqrt(1 + y * y))
        + y * np.sqrt(1 + x * x) * np.arctan(y / np.sqrt(1 + x * x))
        - x * np.arctan(x) - y * np.arctan(y))


def _corner(x, y, eta, zeta):
    u = y - eta
    s = x * x + zeta * zeta
    r = np.sqrt(s)
    q = s + u * u
    at = u * r * np.arctan(u / r) if r > 0 else 0.0
    lg = 0.25 * (s - u * u) * np.log(q) if q > 0 else 0.0
    return at - lg


def ff_perpendicular(x1, x2, y1, y2, eta1, eta2, zeta1, zeta2):
    """F from [x1,x2] x [y1,y2] in z = 0 to [eta1,eta2] (y) x [zeta1,zeta2] (z) in x = 0."""
    tot = 0.0
    for (i, x), (j, y), (k, e), (m, z) in itertools.product(enumerate((x1, x2)), enumerate((y1, y2)),
                                                            enumerate((eta1, eta2)), enumerate((zeta1, zeta2))):
        tot += (-1) ** (i + j + k + m) * _corner(x, y, e, z)
    return tot / (2 * np.pi * (x2 - x1) * (y2 - y1))


def parallel_cases():
    """(points, normals, exact) of tests/test_universal_formfactor.py:11-45."""
    out = []
    for h, d in itertools.product([1.0, 2.0, 3.0, 4.0], [1.0, 2.0, 3.0, 4.0]):
        w = 1.0
        p1 = [[0, 0, 0], [w, 0, 0], [w, 0, h], [0, 0, h]]
        p2 = [[0, d, 0], [0, d, h], [w, d, h], [w, d, 0]]
        out.append(([p1, p2], [[0, 1, 0], [0, -1, 0]], ff_parallel(w, h, d)))
    return out


def common_edge_cases():
    """tests/test_universal_formfactor.py:48-88: vertical h x l patch -> floor w x l patch."""
    out = []
    for w, h in itertools.product([1.0, 2.0, 3.0], [1.0, 2.0, 3.0]):
        ln = 1.0
        p1 = [[0, 0, 0], [0, ln, 0], [0, ln, h], [0, 0, h]]
        p2 = [[0, 0, 0], [w, 0, 0], [w, ln, 0], [0, ln, 0]]
        exact = ff_perpendicular(0, w, 0, ln, 0, ln, 0, h) * (w * ln) / (h * ln)  # reciprocity
        out.append(([p1, p2], [[1, 0, 0], [0, 0, 1]], exact))
    return out


def common_vertex_cases():
    """tests/test_universal_formfactor.py:91-135: floor w2 x l2 -> wall w1 x l1 touching at the origin."""
    out = []
    for w1, l1, w2, l2 in itertools.product([1.0, 2.0, 3.0], repeat=4):
        p1 = [[0, 0, 0], [w2, 0, 0], [w2, l2, 0], [0, l2, 0]]
        p2 = [[0, 0, 0], [0, 0, w1], [0, -l1, w1], [0, -l1, 0]]
        out.append(([p1, p2], [[0, 0, 1], [1, 0, 0]], ff_perpendicular(0, w2, 0, l2, -l1, 0, 0, w1)))
    return out


FF_CASES = {"parallel": (parallel_cases, 1.5), "common_edge": (common_edge_cases, 2.0),
            "common_vertex": (common_vertex_cases, 5.0)}


def _stack(cases):
    pts = np.array([p for c in cases for p in c[0]], dtype=float)
    normals = np.array([nv for c in cases for nv in c[1]], dtype=float)
    pairs = np.array([[2 * k, 2 * k + 1] for k in range(len(cases))], dtype=np.int32)
    exact = np.array([c[2] for c in cases])
    return pts, normals, pairs, exact


def test_corner_sum_reproduces_common_edge_closed_form():
    """The general perpendicular formula against Howell C-14 (common edge), to rounding."""
    for w, h, ln in [(1.0, 1.0, 1.0), (2.0, 3.0, 1.0), (3.0, 1.0, 2.0)]:
        big_w, big_h = w / ln, h / ln
        r = np.sqrt(big_w ** 2 + big_h ** 2)
        t = big_w * np.arctan(1 / big_w) + big_h * np.arctan(1 / big_h) - r * np.arctan(1 / r)
        g = (np.log((1 + big_w ** 2) * (1 + big_h ** 2) / (1 + r ** 2))
             + big_w ** 2 * np.log(big_w ** 2 * (1 + r ** 2) / ((1 + big_w ** 2) * r ** 2))
             + big_h ** 2 * np.log(big_h ** 2 * (1 + r ** 2) / ((1 + big_h ** 2) * r ** 2)))
        c14 = (t + g / 4) / (np.pi * big_w)
        np.testing.assert_allclose(ff_perpendicular(0, w, 0, ln, 0, ln, 0, h), c14, rtol=1e-13)


@pytest.mark.parametrize("kind", sorted(FF_CASES))
def test_oracle_form_factors_vs_analytic(kind):
    from oracle import oracle as orc
    make, tol_percent = FF_CASES[kind]
    pts, normals, pairs, exact = _stack(make())
    ff = np.asarray(orc.form_factors(pts, normals, orc.areas(pts), pairs))
    got = ff[pairs[:, 0], pairs[:, 1]] if ff.ndim == 2 else ff
    assert np.max(100 * np.abs(got - exact) / exact) < tol_percent


# ------------------------------------------------------------------ GPU helpers


def _dev(a, dtype):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def _stream():
    import torch
    return torch.cuda.current_stream().cuda_stream


def gpu_form_factors(pts, normals, areas, pairs, precision):
    """sp_form_factors on device copies of the inputs; FP64 result per pair."""
    import torch
    from sparrowpy_gb300 import _native as nat
    n, m = len(pts), len(pairs)
    ff = torch.zeros((m,), dtype=torch.float64, device="cuda")
    method = torch.zeros((m,), dtype=torch.uint8, device="cuda")
    wsz = nat.size("sp_form_factors_workspace", n, m)
    ws = torch.empty((max(wsz, 1),), dtype=torch.uint8, device="cuda")
    p, nr, ar, pr = (_dev(pts, torch.float64), _dev(normals, torch.float64), _dev(areas, torch.float64),
                     _dev(pairs, torch.int32))
    nat.call("sp_form_factors", nat.SP_F32 if precision == "fp32" else nat.SP_F64, n, np.asarray(pts).shape[1], m,
             pr.data_ptr(),
             p.data_ptr(), nr.data_ptr(), ar.data_ptr(), ff.data_ptr(), method.data_ptr(), ws.data_ptr(), wsz,
             _stream())
    return ff.cpu().numpy()


def _quad_area(p):
    p = np.asarray(p, dtype=float)
    return 0.5 * np.linalg.norm(np.cross(p[1] - p[0], p[2] - p[0])) + \
        0.5 * np.linalg.norm(np.cross(p[2] - p[0], p[3] - p[0]))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("kind", sorted(FF_CASES))
def test_gpu_form_factors_vs_analytic(kind, precision):
    make, tol_percent = FF_CASES[kind]
    pts, normals, pairs, exact = _stack(make())
    areas = np.array([_quad_area(p) for p in pts])
    got = gpu_form_factors(pts, normals, areas, pairs, precision)
    assert np.max(100 * np.abs(got - exact) / exact) < tol_percent


@pytest.mark.gpu
@pytest.mark.parametrize("width", [1.0, 2.0, 3.0, 4.0])
def test_reciprocity_with_different_areas(width):
    """F'(i -> j) = F_ij for i < j and F_ji A_j / A_i for i > j (RadiosityFast.py:1255-1256).

    The stated areas [w, 1, 1, w] are the reference test's, not the patches'
    own, so the relation is checked on the numbers the kernel was given.
    """
    import torch
    from sparrowpy_gb300 import _native as nat
    w = width
    p1 = [[0., 0., 0.], [w, 0., 0.], [w, 1., 0.], [0., 1., 0.]]
    p2 = [[0., 0., 1.], [0., 1., 1.], [w, 1., 1.], [w, 0., 1.]]
    pts = np.array([p1, p2, p2, p1])
    normals = np.array([[0., 0., 1.], [0., 0., -1.], [0., 0., -1.], [0., 0., 1.]])
    areas = np.array([w, 1., 1., w])
    centers = np.array([[w / 2, .5, 0.], [.5, .5, 1.], [.5, .5, 1.], [w / 2, .5, 0.]])
    pairs = np.array([[0, 1], [2, 3]], dtype=np.int32)
    ff = gpu_form_factors(pts, normals, areas, pairs, "fp64")
    pair_index = np.full((4, 4), -1, dtype=np.int32)
    pair_index[0, 1], pair_index[2, 3] = 0, 1
    src = np.array([0, 1, 2, 3], dtype=np.int32)
    dst = np.array([1, 0, 3, 2], dtype=np.int32)
    n_dir = len(src)
    outs = {k: torch.empty((n_dir,), dtype=torch.float64, device="cuda") for k in ("dist", "unit", "fp")}
    idx = {k: torch.empty((n_dir,), dtype=torch.int32, device="cuda") for k in ("out", "in")}
    keep = [_dev(src, torch.int32), _dev(dst, torch.int32), _dev(centers, torch.float64),
            _dev(areas, torch.float64), _dev(pair_index, torch.int32), _dev(ff, torch.float64),
            _dev(np.array([0, 1, 1, 0]), torch.int32)]
    nat.call("sp_pair_setup", n_dir, 4, *[t.data_ptr() for t in keep[:6]], keep[6].data_ptr(), 0, None, 0, None,
             idx["out"].data_ptr(), idx["in"].data_ptr(), outs["dist"].data_ptr(), outs["unit"].data_ptr(),
             outs["fp"].data_ptr(), _stream())
    fp = outs["fp"].cpu().numpy()
    f01, f10, f23, f32 = fp
    assert f01 == ff[0] and f23 == ff[1]
    assert f10 == ff[0] * areas[0] / areas[1]  # same operation order: bit-exact
    assert f32 == ff[1] * areas[2] / areas[3]
    np.testing.assert_allclose(f10 / w, f01, rtol=2e-16)
    np.testing.assert_allclose(f23 / w, f32, rtol=2e-16)
    assert abs(f01 - f32) < 1e-9
    assert abs(f23 - f10) < 1e-9


# ------------------------------------------------------------- room-level cases


@pytest.mark.gpu
@pytest.mark.parametrize("xyz", [(2.0, 1.0, 2.0), (2.0, 2.0, 2.0), (3.0, 1.0, 2.0), (3.0, 2.0, 2.0)])
def test_ff_tilde_energy_conservation(xyz):
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.geometry import shoebox_room_stub
    r = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(*xyz), 1.0, precision="fp64")
    r.bake_geometry()
    fft = r._form_factors_tilde
    n = r.n_patches
    assert (n - np.sum(fft)) / n < 1e-2
    for i in range(n):
        assert 1 - np.sum(fft[i]) < 1e-2


@pytest.mark.gpu
def test_cube_visibility_pattern():
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.geometry import shoebox_room_stub
    r = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(1, 1, 1), 0.5)
    r.bake_geometry()
    v = r._visibility_matrix
    assert v.shape == (24, 24)
    for i in range(6):
        k = 4 * i
        assert not v[k + 4:, k:k + 4].any()
        assert v[k:k + 4, k + 4:].all()
    assert v.sum() == 24 ** 2 - 21 * 4 ** 2


def equal_angle_upper(delta_deg):
    """Equal-angle grid (colatitude x azimuth, poles repeated per azimuth) with elevation >= 0."""
    from sparrowpy_gb300.coords import Coordinates
    col = np.deg2rad(np.arange(0, 90 + delta_deg / 2, delta_deg))
    az = np.deg2rad(np.arange(0, 360, delta_deg))
    cc, aa = np.meshgrid(col, az, indexing="ij")
    xyz = np.stack([np.sin(cc) * np.cos(aa), np.sin(cc) * np.sin(aa), np.cos(cc)], axis=-1).reshape(-1, 3)
    return Coordinates.from_cartesian(xyz, weights=np.ones(xyz.shape[0]))


@pytest.mark.gpu
def test_outgoing_direction_map_of_perpendicular_walls():
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering
    from sparrowpy_gb300.coords import FrequencyData
    from sparrowpy_gb300.geometry import Polygon
    walls = [Polygon([[0, 0, 0], [0, 1, 0], [0, 1, 1], [0, 0, 1]], normal=[1, 0, 0], up_vector=[0, 0, 1]),
             Polygon([[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]], normal=[0, 1, 0], up_vector=[0, 0, -1])]
    r = DirectionalRadiosityFast.from_polygon(walls, 1)
    dirs = equal_angle_upper(45)
    f = np.array([1000.0])
    brdf = create_from_scattering(dirs, dirs, FrequencyData(0.5 * np.ones_like(f), f),
                                  FrequencyData(0.1 * np.ones_like(f), f))
    r.set_wall_brdf(np.arange(2), brdf, dirs, dirs)
    r.bake_geometry()
    p2o = r._patch_2_brdf_outgoing_index
    n_out = dirs.csize
    assert p2o.ndim == 2 and p2o.shape == (r.n_patches, r.n_patches)
    assert p2o[0, 0] == n_out and p2o[1, 1] == n_out
    i0, i1 = p2o[0, 1], p2o[1, 0]
    assert i0 == i1  # the flipped up vectors mirror the walls over the plane x = y
    v0 = np.asarray(r._brdf_outgoing_directions[0].cartesian).reshape(-1, 3)[int(i0)]
    v1 = np.asarray(r._brdf_outgoing_directions[1].cartesian).reshape(-1, 3)[int(i1)]
    np.testing.assert_allclose([v0[2], v1[2]], 0, atol=1e-7)
    np.testing.assert_allclose(v0, -v1, atol=1e-7)


def _plane_ratio(source, receiver, precision):
    """Diffuse / specular energy of a 20 x 20 m Lambertian plane at order 0 (no bake)."""
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    from sparrowpy_gb300.geometry import Polygon
    src, rcv = np.asarray(source, float), np.asarray(receiver, float)
    image = src * np.array([1, 1, -1])
    reflection_len = np.linalg.norm(rcv - image)
    plane = Polygon([[-10, -10, 0], [10, -10, 0], [10, 10, 0], [-10, 10, 0]], [1, 0, 0], [0, 0, 1])
    r = DirectionalRadiosityFast.from_polygon([plane], 1, precision=precision)
    one = Coordinates(0, 0, 1, weights=1)
    brdf = create_from_scattering(one, one, FrequencyData(1, [100]), FrequencyData(0, [100]))
    r.set_wall_brdf(np.arange(1), brdf, one, one)
    r.set_air_attenuation(FrequencyData(np.zeros(1), np.array([100.0])))
    r.init_source_energy(Coordinates(*src))
    r.calculate_energy_exchange(speed_of_sound=343, etc_time_resolution=1.0, etc_duration=1,
                                max_reflection_order=0)
    diffuse = r.collect_energy_receiver_mono(Coordinates(*rcv))
    return np.sum(diffuse.time) / (1 / (4 * np.pi * reflection_len ** 2))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("source,receiver", [((0, 0, 3), (0, 0, 3)), ((0, 0, 5), (0, 0, 3))])
def test_infinite_diffuse_plane_on_normal(source, receiver, precision):
    """Svensson's cases 1 and 2: the ratio tends to 2; the finite plane gives slightly less."""
    ratio = _plane_ratio(source, receiver, precision)
    assert ratio < 2
    np.testing.assert_allclose(ratio, 1.97, rtol=0.01)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("theta_deg", [30, 45, 60])
def test_infinite_diffuse_plane_same_height(theta_deg, precision):
    """Svensson's case 3: the ratio is 2 cos(theta) for the specular incidence angle theta."""
    th = np.deg2rad(theta_deg)
    source = (2 * np.sin(th), 0.0, 2 * np.cos(th))
    receiver = (-2 * np.sin(th), 0.0, 2 * np.cos(th))
    ratio = _plane_ratio(source, receiver, precision)
    np.testing.assert_allclose(ratio, 2 * np.cos(th), atol=0.03, rtol=0.03)


def _diffuse_room(walls, patch_size, freqs, absorption, precision):
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    r = DirectionalRadiosityFast.from_polygon(walls, patch_size, precision=precision)
    one = Coordinates(0, 0, 1, weights=1)
    brdf = create_from_scattering(one, one, FrequencyData(np.ones(freqs.size), freqs),
                                  FrequencyData(np.zeros(freqs.size) + absorption, freqs))
    r.set_wall_brdf(np.arange(len(walls)), brdf, one, one)
    r.set_air_attenuation(FrequencyData(np.zeros_like(freqs, dtype=float), freqs))
    r.bake_geometry()
    return r


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("ps", [1, 1.5])
@pytest.mark.parametrize("order", [10, 20])
@pytest.mark.parametrize("rec", [(0.5, 1, 2.5), (1, 2.5, 1.5)])
def test_reciprocity_shoebox(rec, order, ps, precision):
    from sparrowpy_gb300.coords import Coordinates
    from sparrowpy_gb300.geometry import shoebox_room_stub
    src = (2, 1.5, 1.5)
    walls = shoebox_room_stub(3, 3, 3)
    etcs = []
    for a, b in ((src, rec), (rec, src)):
        r = _diffuse_room(walls, ps, np.array([1000.0]), 0.0, precision)
        r.init_source_energy(Coordinates(*a))
        r.calculate_energy_exchange(speed_of_sound=343, etc_time_resolution=1 / 200, etc_duration=0.5,
                                    max_reflection_order=order)
        etcs.append(r.collect_energy_receiver_mono(Coordinates(*b)).time[0])
    np.testing.assert_array_almost_equal(np.sum(etcs[1]), np.sum(etcs[0]))
    np.testing.assert_array_almost_equal(etcs[1], etcs[0])


@pytest.mark.gpu
@pytest.mark.parametrize("src", [(2., 0, 0), (2., 2., 0), (2., 0., 2.)])
@pytest.mark.parametrize("rec", [(1., 0., 0), (2., -2., 0), (2., 0., -2.)])
def test_reciprocity_source_patch_receiver(src, rec):
    """e_s(source -> patch) * e_r(patch -> receiver) is symmetric in source and receiver."""
    import torch
    from sparrowpy_gb300 import _native as nat
    pts = np.array([[[0, -1, -1], [0, -1, 1], [0, 1, 1], [0, 1, -1]]], dtype=float)
    centers = pts.mean(axis=1)
    ones = dict(vis=_dev(np.ones(1), torch.uint8), wall=_dev(np.zeros(1), torch.int32),
                slot=_dev(np.zeros(1), torch.int32), dirs=_dev(np.array([[[0, 0, 1.0]]]), torch.float64),
                brdf=_dev(np.ones((1, 1, 1, 1)), torch.float64), att=_dev(np.zeros(1), torch.float64))
    p, c = _dev(pts, torch.float64), _dev(centers, torch.float64)
    energy = []
    for a, b in ((src, rec), (rec, src)):
        e0 = torch.empty((1, 1), dtype=torch.float64, device="cuda")
        d0 = torch.empty((1,), dtype=torch.float64, device="cuda")
        e0dir = torch.empty((1, 1, 1), dtype=torch.float64, device="cuda")
        sa = _dev(np.asarray(a, float), torch.float64)
        nat.call("sp_source_energy", sa.data_ptr(), 1, c.data_ptr(), p.data_ptr(), 4, ones["vis"].data_ptr(), 1,
                 ones["att"].data_ptr(), ones["wall"].data_ptr(), ones["slot"].data_ptr(), 1, ones["dirs"].data_ptr(),
                 1, ones["brdf"].data_ptr(), e0.data_ptr(), d0.data_ptr(), e0dir.data_ptr(), _stream())
        rb = _dev(np.asarray(b, float), torch.float64)
        rfac = torch.empty((1,), dtype=torch.float64, device="cuda")
        ridx = torch.empty((1,), dtype=torch.int32, device="cuda")
        dist = torch.empty((1,), dtype=torch.float64, device="cuda")
        nat.call("sp_receiver_factors", rb.data_ptr(), 1, c.data_ptr(), p.data_ptr(), 4, ones["vis"].data_ptr(),
                 ones["wall"].data_ptr(), 1, ones["dirs"].data_ptr(), rfac.data_ptr(), ridx.data_ptr(),
                 dist.data_ptr(), _stream())
        energy.append(e0.cpu().numpy()[:, 0] * rfac.cpu().numpy())
    assert energy[0][0] > 0
    np.testing.assert_array_almost_equal(energy[0], energy[1])


@pytest.mark.gpu
@pytest.mark.parametrize("freqs", [np.array([1000.0]), np.array([500.0, 1000.0, 2000.0])])
def test_multi_receiver_equals_single_receivers(freqs):
    from sparrowpy_gb300.coords import Coordinates
    from sparrowpy_gb300.geometry import shoebox_room_stub
    r = _diffuse_room(shoebox_room_stub(1, 1, 1), 0.2, freqs, 0.1, "fp32")
    r.init_source_energy(Coordinates(.5, .5, .5))
    r.calculate_energy_exchange(speed_of_sound=343, etc_time_resolution=1 / 100, etc_duration=1.0,
                                max_reflection_order=10)
    receivers = Coordinates([.25, .45, .75], [.45, .45, .45], [.75, .75, .75])
    big = r.collect_energy_receiver_mono(receivers)
    assert big.cshape[0] == 3 and big.cshape[1] == freqs.size
    for i in range(3):
        small = r.collect_energy_receiver_mono(Coordinates(*receivers.cartesian.reshape(-1, 3)[i]))
        np.testing.assert_array_almost_equal(big.time[i], small.time[0])


@pytest.mark.gpu
def test_source_visibility():
    """A source outside the closed cube sees no patch; one inside sees all (no bake needed)."""
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.coords import Coordinates
    from sparrowpy_gb300.geometry import shoebox_room_stub
    r = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(1, 1, 1), patch_size=1.)
    r.init_source_energy(Coordinates(3., 3., 3.))
    np.testing.assert_equal(r._energy_init_source, np.zeros_like(r._energy_init_source))
    np.testing.assert_equal(r._source_visibility, np.zeros_like(r._source_visibility))
    r.init_source_energy(Coordinates(.5, .5, .5))
    np.testing.assert_equal(r._source_visibility, np.ones_like(r._source_visibility))
    assert (r._energy_init_source != 0).any()


@pytest.mark.gpu
def test_receiver_visibility_default_order():
    """Default max_reflection_order (-1): the source energy only, without bake_geometry()."""
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.coords import Coordinates
    from sparrowpy_gb300.geometry import shoebox_room_stub
    r = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(1, 1, 1), patch_size=1.)
    r.init_source_energy(Coordinates(.5, .5, .5))
    r.calculate_energy_exchange(speed_of_sound=343, etc_time_resolution=.2, etc_duration=1.)
    etc = r.collect_energy_receiver_mono(Coordinates([3., -5., .5], [3., 5., .5], [3., 4., .5]))
    np.testing.assert_equal(etc.time[0:2, 0, :], np.zeros((2, 5)))
    assert (etc.time[-1, 0, :] != 0).any()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_plane_without_visible_pairs_keeps_source_energy(precision):
    """No patch sees another: every order adds nothing to the source energy (edge case)."""
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    from sparrowpy_gb300.geometry import Polygon
    plane = Polygon([[-2, -2, 0], [2, -2, 0], [2, 2, 0], [-2, 2, 0]], [1, 0, 0], [0, 0, 1])
    one = Coordinates(0, 0, 1, weights=1)
    f = np.array([500.0, 1000.0])
    out = []
    for order, bake in ((0, False), (5, True)):
        r = DirectionalRadiosityFast.from_polygon([plane], 1, precision=precision)
        r.set_wall_brdf(np.arange(1), create_from_scattering(one, one, FrequencyData(np.ones(2), f),
                                                             FrequencyData(np.full(2, 0.2), f)), one, one)
        r.set_air_attenuation(FrequencyData(np.zeros(2), f))
        if bake:
            r.bake_geometry()
            assert r._visible_patches.shape[0] == 0
        r.init_source_energy(Coordinates(0.3, -0.4, 2.0))
        r.calculate_energy_exchange(343, 1e-3, 0.05, order)
        out.append(r.collect_energy_receiver_mono(Coordinates(-0.5, 0.7, 1.5)).time)
    assert np.sum(out[0]) > 0
    np.testing.assert_array_equal(out[0], out[1])


@pytest.mark.gpu
def test_source_delay_beyond_histogram_raises_index_error():
    """The reference writes E0 at bin int(d0 / c / dt) (RadiosityFast.py:1037-1070); past the end: IndexError."""
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.coords import Coordinates
    from sparrowpy_gb300.geometry import shoebox_room_stub
    r = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(1, 1, 1), 0.5)
    r.bake_geometry()
    r.init_source_energy(Coordinates(0.5, 0.5, 0.5))
    with pytest.raises(IndexError):
        r.calculate_energy_exchange(343, 1e-3, 1e-3, 2, recalculate=True)  # one bin; delays are >= 1 bin


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_long_histogram_takes_dense_exchange(precision):
    """More than 65535 bins: the structured kernels' 16-bit delays do not reach; "auto" runs the dense
    exchange, which matches the oracle (rel L2 <= 1e-10 FP64, 1e-4 FP32)."""
    from conftest import load_golden, radiosity_from_golden, rel_l2, scene_from_golden
    from oracle import oracle as orc
    from sparrowpy_gb300.coords import Coordinates
    g = load_golden("cube")
    c, dt, duration, k = 343.0, 1e-5, 0.7, 2  # 70000 bins
    ref = orc.solve(scene_from_golden(g), g["source"], np.atleast_2d(g["receivers"]), c, dt, duration, k)
    r = radiosity_from_golden(g, precision)
    r.bake_geometry()
    r.init_source_energy(Coordinates(*g["source"]))
    r.calculate_energy_exchange(c, dt, duration, k)
    assert r.exchange_stats["algorithm"] == "dense"
    rcv = np.atleast_2d(g["receivers"])
    mono = r.collect_energy_receiver_mono(Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])).time
    assert rel_l2(mono, ref["mono"]) <= (1e-10 if precision == "fp64" else 1e-4)
    with pytest.raises(ValueError):
        r.calculate_energy_exchange(c, dt, duration, k, recalculate=True, algorithm="structured")
