"""The directional Kang solver (sparrowpy/classes/RadiosityKang.py:500-810, :1059-1202;
tests/test_RadiosityDirectional.py).

The reference's own tests and stored results, restated:
* directional data replaced by ones: the init equals the stored plain init
  (reference_matrix_directional_patch_size*.far) for every band and
  direction, and the 10 x 20 x 15 m simulation equals the stored one
  (simulation_X10_k*_5m.far) to 4 decimals, also after write / from_read;
* the specular data of specular_gaussian5.sofa on two perpendicular cube
  walls gives the stored (all zero) response to 4 decimals, for 24 wall
  pairs and two patch sizes;
* to_dict / from_dict round trips.
The SOFA files' arrays come from tests/golden/sofa.npz (make_sofa_golden.py);
the stored results from tests/golden/kang.npz.  The oracle (oracle/kang.py)
is pinned to the same results on the CPU, and the GPU is checked against the
oracle on a seeded room with random tables, two bands and air attenuation
(1e-12 relative).
"""
import numpy as np
import numpy.testing as npt
import pytest

from conftest import load_golden
from oracle import kang as ok
from sparrowpy_gb300.coords import FrequencyData
from sparrowpy_gb300.geometry import Polygon, shoebox_room_stub
from sparrowpy_gb300.sofa import sofa_pos
from test_kang import GOLD, rel
from test_sofa import ihta_data

PERPENDICULAR = [[0, 2], [0, 4], [2, 0], [2, 4], [4, 0], [4, 2], [1, 2], [1, 3], [1, 4], [1, 5], [2, 1], [2, 5],
                 [0, 3], [0, 5], [3, 0], [3, 1], [3, 4], [3, 5], [4, 1], [4, 3], [5, 0], [5, 1], [5, 2], [5, 3]]


@pytest.fixture(scope="module")
def sofa_gold():
    return load_golden("sofa")


def specular_data(g):
    data = FrequencyData(g["specular_gaussian5_data"], g["specular_gaussian5_N"])
    src = sofa_pos(str(g["specular_gaussian5_source_type"]), g["specular_gaussian5_source_position"])
    rcv = sofa_pos(str(g["specular_gaussian5_receiver_type"]), g["specular_gaussian5_receiver_position"])
    src.weights, rcv.weights = g["specular_gaussian5_source_weights"], g["specular_gaussian5_receiver_weights"]
    return data, src, rcv


def oracle_wall(wall, size, other, data, src, rcv, absorption=None, attenuation=None):
    """An oracle wall dict with directional data as PatchesDirectionalKang builds it."""
    nb = data.frequencies.size
    return dict(pts=np.asarray(wall.pts, float), normal=np.asarray(wall.normal, float), max_size=size, other=other,
                scattering=np.ones(nb), absorption=np.full(nb, 0.1) if absorption is None else np.asarray(absorption),
                attenuation=np.zeros(nb) if attenuation is None else np.asarray(attenuation),
                patches=ok.kang_patches(wall.pts, size), dir_data=np.abs(np.asarray(data.freq)) * np.pi,
                dir_sources=ok.reference_frame_directions(src.cartesian, wall.normal, wall.up_vector),
                dir_receivers=ok.reference_frame_directions(rcv.cartesian, wall.normal, wall.up_vector))


def x10_polygons():
    X, Y, Z = 10, 20, 15
    return [Polygon([[0, 0, 0], [X, 0, 0], [X, Y, 0], [0, Y, 0]], [1, 0, 0], [0, 0, 1]),
            Polygon([[0, 0, 0], [X, 0, 0], [X, 0, Z], [0, 0, Z]], [1, 0, 0], [0, 1, 0]),
            Polygon([[0, Y, 0], [X, Y, 0], [X, Y, Z], [0, Y, Z]], [1, 0, 0], [0, -1, 0])]


# ------------------------------------------------------------------ oracle, CPU
@pytest.mark.parametrize("size", [0.5, 1])
def test_oracle_directional_omni_init(sofa_gold, size):
    """test_RadiosityDirectional.py:149-179 on the oracle: data of ones gives the stored plain init."""
    data, src, rcv = ihta_data(sofa_gold)
    for i, wall in enumerate(shoebox_room_stub(1, 1, 1)):
        w = oracle_wall(wall, size, [], data, src, rcv)
        w["dir_data"] = np.ones_like(w["dir_data"])
        E = ok.dkang_init(w, 3, 5, [0.5, 0.5, 0.5], 1.0, 1000, 346.18)
        for b in range(E.shape[0]):
            for d in range(E.shape[-1]):
                npt.assert_almost_equal(GOLD[f"E_init_size{size:g}"][0], E[b, ..., d])


@pytest.mark.parametrize("k", [2, 3])
def test_oracle_directional_x10(sofa_gold, k):
    """test_RadiosityDirectional.py:16-62 on the oracle, with its tolerance (4 decimals)."""
    data, src, rcv = ihta_data(sofa_gold)
    polys = x10_polygons()
    walls = [oracle_wall(p, 5, [j for j in range(3) if j != i], data, src, rcv) for i, p in enumerate(polys)]
    for w in walls:
        w["dir_data"] = np.ones_like(w["dir_data"])
    E, _ = ok.dkang_run(walls, k, 5, [10, 6, 1], 343, 50)
    ir = ok.dkang_energy_at_receiver(walls, E, k, [20, 2, 1], [10, 6, 1], 343, 50)
    ir = ir / np.max(np.abs(ir))
    for b in range(ir.shape[0]):
        npt.assert_almost_equal(GOLD[f"sim_X10_k{k}_time"][0], ir[b], decimal=4)


@pytest.mark.parametrize("size", [0.5, 1])
def test_oracle_directional_specular(sofa_gold, size):
    """test_RadiosityDirectional.py:182-238 on the oracle: the stored response is zero (4 decimals)."""
    data, src, rcv = specular_data(sofa_gold)
    walls = shoebox_room_stub(1, 1, 1)
    for a, b in PERPENDICULAR[:6]:
        pair = [oracle_wall(walls[a], size, [1], data, src, rcv), oracle_wall(walls[b], size, [0], data, src, rcv)]
        E, _ = ok.dkang_run(pair, 3, 5, [0.5, 0.5, 0.5], 346.18, 1000)
        ir = ok.dkang_receiver(pair[0], E[0], 3, [0.5, 0.5, 0.5], 346.18, 1000) + \
            ok.dkang_receiver(pair[1], E[1], 3, [0.5, 0.5, 0.5], 346.18, 1000)
        npt.assert_almost_equal(np.zeros((1, 5000)), ir, decimal=4)


# --------------------------------------------------------------------- GPU
def gpu_directional(wall, size, other, wall_id, data, src, rcv, **kw):
    from sparrowpy_gb300.kang import PatchesDirectionalKang
    return PatchesDirectionalKang(wall, size, other, wall_id, data, src, rcv, **kw)


@pytest.mark.gpu
@pytest.mark.parametrize("size", [0.5, 1])
def test_gpu_directional_omni_init(sofa_gold, size):
    """test_RadiosityDirectional.py:149-179: data of ones gives the stored plain init for every band and
    direction (stored to 7 decimals in the reference; here 1e-12 relative, as the plain init)."""
    from sparrowpy_gb300.sound_object import SoundSource
    data, src, rcv = ihta_data(sofa_gold)
    source = SoundSource([0.5, 0.5, 0.5], [0, 1, 0], [0, 0, 1])
    for wall in shoebox_room_stub(1, 1, 1):
        p = gpu_directional(wall, size, [], 0, data, src, rcv)
        p.directivity_data.freq = np.ones_like(p.directivity_data.freq)
        p.init_energy_exchange(3, 5, source, 1000, 346.18)
        E = p.E_matrix
        assert E.shape == (5, 4, len(p.patches), 5000, 36)
        for b in range(E.shape[0]):
            for d in range(E.shape[-1]):
                npt.assert_allclose(E[b, ..., d], GOLD[f"E_init_size{size:g}"][0], rtol=1e-12, atol=1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("k", [2, 3])
def test_gpu_directional_x10(sofa_gold, k, tmp_path):
    """test_RadiosityDirectional.py:16-121: the simulation with data of ones, to 4 decimals against the
    stored result for every band, before and after write / from_read; and the oracle to 1e-12."""
    import sparrowpy_gb300 as sp
    from sparrowpy_gb300.sound_object import Receiver, SoundSource
    data, src, rcv = ihta_data(sofa_gold)
    polys = x10_polygons()
    walls = [gpu_directional(p, 5, [j for j in range(3) if j != i], i, data, src, rcv) for i, p in enumerate(polys)]
    radi = sp.DirectionalRadiosityKang(walls, 5, k, 5, None, speed_of_sound=343, sampling_rate=50)
    for p in radi.patch_list:
        p.directivity_data.freq = np.ones_like(p.directivity_data.freq)
    radi.run(SoundSource([10, 6, 1], [0, 1, 0], [0, 0, 1]))
    receiver = Receiver([20, 2, 1], [0, 1, 0], [0, 0, 1])
    ir = radi.energy_at_receiver(receiver)
    norm = ir / np.max(np.abs(ir))
    for b in range(norm.shape[0]):
        npt.assert_almost_equal(GOLD[f"sim_X10_k{k}_time"][0], norm[b], decimal=4)
    radi.write(tmp_path / "radiosity.far")
    back = sp.DirectionalRadiosityKang.from_read(tmp_path / "radiosity.far")
    npt.assert_array_equal(back.energy_at_receiver(receiver), ir)
    owalls = [oracle_wall(p, 5, [j for j in range(3) if j != i], data, src, rcv) for i, p in enumerate(polys)]
    for w in owalls:
        w["dir_data"] = np.ones_like(w["dir_data"])
    E, _ = ok.dkang_run(owalls, k, 5, [10, 6, 1], 343, 50)
    for p, e in zip(radi.patch_list, E):
        assert rel(p.E_matrix, e) < 1e-12
    assert rel(ir, ok.dkang_energy_at_receiver(owalls, E, k, [20, 2, 1], [10, 6, 1], 343, 50)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("size", [0.5, 1])
def test_gpu_directional_specular(sofa_gold, size):
    """test_RadiosityDirectional.py:182-238: 24 perpendicular wall pairs with the specular data; the
    stored response is zero (4 decimals); the oracle to 1e-12 of the largest histogram value."""
    from sparrowpy_gb300.sound_object import Receiver, SoundSource
    data, src, rcv = specular_data(sofa_gold)
    walls = shoebox_room_stub(1, 1, 1)
    source = SoundSource([0.5, 0.5, 0.5], [0, 1, 0], [0, 0, 1])
    receiver = Receiver([0.5, 0.5, 0.5], [0, 1, 0], [0, 0, 1])
    for n_pair, (a, b) in enumerate(PERPENDICULAR):
        p1 = gpu_directional(walls[a], size, [1], 0, data, src, rcv)
        p2 = gpu_directional(walls[b], size, [0], 1, data, src, rcv)
        patches = [p1, p2]
        for p in patches:
            p.calculate_form_factor(patches)
            p.init_energy_exchange(3, 5, source, 1000, 346.18)
        for k in range(1, 4):
            p1.calculate_energy_exchange(patches, k, 346.18, 1000)
            p2.calculate_energy_exchange(patches, k, 346.18, 1000)
        ir = p1.energy_at_receiver(3, receiver, speed_of_sound=346.18, sampling_rate=1000) + \
            p2.energy_at_receiver(3, receiver, speed_of_sound=346.18, sampling_rate=1000)
        npt.assert_almost_equal(np.zeros((1, 5000)), ir, decimal=4)
        if n_pair < 4:
            pair = [oracle_wall(walls[a], size, [1], data, src, rcv), oracle_wall(walls[b], size, [0], data, src, rcv)]
            E, _ = ok.dkang_run(pair, 3, 5, [0.5, 0.5, 0.5], 346.18, 1000)
            for p, e in zip(patches, E):
                scale = max(np.abs(e).max(), 1e-300)
                assert np.abs(p.E_matrix - e).max() <= 1e-12 * scale


@pytest.mark.gpu
def test_gpu_directional_random_room_vs_oracle():
    """A 3 x 2 x 2 m room, 0.5 m patches, two bands with air attenuation and per-wall absorption, seeded
    random data over 14 incoming and 10 outgoing directions: E of every wall and the receiver response
    against the oracle, 1e-12 relative."""
    import sparrowpy_gb300 as sp
    from sparrowpy_gb300.coords import Coordinates
    from sparrowpy_gb300.sound_object import Receiver, SoundSource
    rng = np.random.default_rng(11)

    def hemisphere(n):
        v = rng.normal(size=(n, 3))
        v[:, 2] = np.abs(v[:, 2]) + 0.05
        return Coordinates.from_cartesian(v / np.linalg.norm(v, axis=1)[:, None], weights=np.full(n, 1.0 / n))

    src, rcv = hemisphere(14), hemisphere(10)
    freqs = np.array([500.0, 1000.0])
    walls = shoebox_room_stub(3, 2, 2)
    n = len(walls)
    absorption = [rng.uniform(0.05, 0.3, 2) for _ in range(n)]
    attenuation = np.array([0.001, 0.004])
    tables = [rng.uniform(0.0, 0.4, (14, 10, 2)) for _ in range(n)]
    patches = [gpu_directional(w, 0.5, [j for j in range(n) if j != i], i, FrequencyData(tables[i], freqs), src, rcv,
                               absorption=absorption[i], sound_attenuation_factor=attenuation)
               for i, w in enumerate(walls)]
    radi = sp.DirectionalRadiosityKang(patches, 0.5, 3, 0.2, None, speed_of_sound=343.0, sampling_rate=1000)
    radi.run(SoundSource([0.7, 0.6, 0.8], [0, 1, 0], [0, 0, 1]))
    ir = radi.energy_at_receiver(Receiver([2.2, 1.3, 1.1], [0, 1, 0], [0, 0, 1]))
    owalls = [oracle_wall(w, 0.5, [j for j in range(n) if j != i], FrequencyData(tables[i], freqs), src, rcv,
                          absorption=absorption[i], attenuation=attenuation) for i, w in enumerate(walls)]
    E, FF = ok.dkang_run(owalls, 3, 0.2, [0.7, 0.6, 0.8], 343.0, 1000)
    for p, e, f in zip(radi.patch_list, E, FF):
        npt.assert_allclose(p.form_factors, f, rtol=1e-12, atol=1e-300)
        assert rel(p.E_matrix, e) < 1e-12
        assert np.count_nonzero(p.E_matrix[:, 1:]) > 0
    ref = ok.dkang_energy_at_receiver(owalls, E, 3, [2.2, 1.3, 1.1], [0.7, 0.6, 0.8], 343.0, 1000)
    assert rel(ir, ref) < 1e-12


@pytest.mark.gpu
def test_gpu_directional_to_from_dict(sofa_gold):
    """test_RadiosityDirectional.py:241-286 (patches) and :289-335 (the solver, also into RadiosityKang)."""
    import sparrowpy_gb300 as sp
    from sparrowpy_gb300.kang import PatchesDirectionalKang
    from sparrowpy_gb300.sound_object import SoundSource
    data, src, rcv = specular_data(sofa_gold)
    wall = shoebox_room_stub(1, 1, 1)[0]
    p = gpu_directional(wall, 0.2, [1], 0, data, src, rcv)
    p.init_energy_exchange(1, 1, SoundSource([0.5, 0.5, 0.5], [0, 1, 0], [0, 0, 1]), 1000, 346.18)
    q = PatchesDirectionalKang.from_dict(p.to_dict())
    npt.assert_array_equal(q.directivity_data.freq, p.directivity_data.freq)
    assert q.directivity_sources == p.directivity_sources
    assert q.directivity_receivers == p.directivity_receivers
    npt.assert_array_equal(q.E_matrix, p.E_matrix)
    assert q.E_n_samples == p.E_n_samples
    for key in ("pts", "up_vector", "normal", "scattering", "absorption", "sound_attenuation_factor"):
        npt.assert_array_equal(getattr(q, key), getattr(p, key))
    assert q.max_size == p.max_size and q.wall_id == p.wall_id
    npt.assert_array_equal(q.other_wall_ids, p.other_wall_ids)

    dsrc, dsrc_s, dsrc_r = ihta_data(sofa_gold)
    walls = [gpu_directional(w, 5, [j for j in range(3) if j != i], i, dsrc, dsrc_s, dsrc_r)
             for i, w in enumerate(x10_polygons())]
    radi = sp.DirectionalRadiosityKang(walls, 5, 3, 5, None, speed_of_sound=343, sampling_rate=50)
    radi.run(SoundSource([10, 6, 1], [0, 1, 0], [0, 0, 1]))
    d = radi.to_dict()
    for cls in (sp.DirectionalRadiosityKang, sp.RadiosityKang):
        back = cls.from_dict(d)
        assert isinstance(back, cls)
        for key in ("patch_size", "max_order_k", "ir_length_s", "speed_of_sound", "sampling_rate"):
            assert getattr(back, key) == getattr(radi, key)
        for a, b in zip(radi.patch_list, back.patch_list, strict=True):
            npt.assert_array_equal(a.E_matrix, b.E_matrix)
            npt.assert_array_equal(a.pts, b.pts)
            assert a.wall_id == b.wall_id and a.max_size == b.max_size
