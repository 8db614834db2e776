"""SOFA files and the directional data read from them (sofa.py, hdf5.py).

tests/golden/sofa.npz holds the arrays of the reference's three SOFA test
files as the package's reader extracts them (make_sofa_golden.py).  They
are pinned by the reference's own known answer: the directivity of
ITA_Dodecahedron.sofa towards a target seen from a rotated source is
0.0001908 (tests/test_radiosity_sound_object.py:21-31 of sparrowpy).  With
the reference tree at hand (SPARROWPY_SRC), the files themselves are read
again and compared with the stored arrays and checksums.
"""
import ast
import hashlib
import os

import numpy as np
import numpy.testing as npt
import pytest

from conftest import load_golden
from sparrowpy_gb300.coords import Coordinates, FrequencyData, cart2sph, sph2cart, unit_radius
from sparrowpy_gb300.sofa import sofa_pos
from sparrowpy_gb300.sound_object import DirectivityMS

SRC = os.environ.get("SPARROWPY_SRC")
FILES = {"ita_dodecahedron": "ITA_Dodecahedron", "ihta": "ihta.E_sec_2",
         "specular_gaussian5": "specular_gaussian5"}


@pytest.fixture(scope="module")
def gold():
    return load_golden("sofa")


def _known_answer(directivity):
    fac = directivity.get_directivity([0, 0, 2], [-0.707106781186548, 0, 0.707106781186548], [0, 1, 0],
                                      [-1, 0, -2], 2)
    npt.assert_almost_equal(fac, 0.0001908)


def test_directivity_known_answer_from_stored_arrays(gold):
    """The reference's test_get_directivity on the extracted directivity (decimal 7, its tolerance)."""
    pos = np.squeeze(gold["ita_dodecahedron_receiver_position"])
    receivers = sofa_pos(str(gold["ita_dodecahedron_receiver_type"]), pos)
    d = DirectivityMS(data=FrequencyData(gold["ita_dodecahedron_data0"], gold["ita_dodecahedron_N"][:4]),
                      receivers=receivers)
    assert d.data.cshape[0] == d.receivers.cshape[0]
    _known_answer(d)


def test_sofa_pos_spherical_and_cartesian():
    """pyfar's _sofa_pos: spherical rows are (azimuth deg, elevation deg, radius)."""
    c = sofa_pos("spherical", np.array([[0.0, 0.0, 2.0], [90.0, 0.0, 1.0], [0.0, 90.0, 3.0], [180.0, -45.0, 1.0]]))
    npt.assert_allclose(c.cartesian, [[2, 0, 0], [0, 1, 0], [0, 0, 3], [-np.sqrt(0.5), 0, -np.sqrt(0.5)]],
                        atol=1e-15)
    assert c.cartesian[1, 0] == 0.0 and c.cartesian[2, 1] == 0.0  # components below eps are zeroed, as pyfar
    npt.assert_array_equal(sofa_pos("cartesian", np.eye(3)).cartesian, np.eye(3))
    with pytest.raises(ValueError):
        sofa_pos("polar", np.eye(3))


def test_unit_radius_round_trip():
    rng = np.random.default_rng(5)
    xyz = rng.normal(size=(50, 3))
    u = unit_radius(xyz)
    npt.assert_allclose(np.linalg.norm(u, axis=1), 1.0, atol=1e-15)
    npt.assert_allclose(u, xyz / np.linalg.norm(xyz, axis=1)[:, None], atol=1e-15)
    az, col, r = cart2sph(*xyz.T)
    npt.assert_allclose(np.stack(sph2cart(az, col, r), axis=1), xyz, atol=1e-14)


def test_directional_walls_rotated_into_their_half_space(gold):
    """The reference's test_init_energy_exchange direction checks (test_RadiosityDirectional.py:124-146):
    after rotation every source and receiver direction of a wall lies on its normal's side."""
    from sparrowpy_gb300.geometry import shoebox_room_stub
    from sparrowpy_gb300.kang import PatchesDirectionalKang
    from oracle import kang as ok
    data, sources, receivers = ihta_data(gold)
    for wall in shoebox_room_stub(1, 1, 1):
        p = PatchesDirectionalKang(wall, 0.2, [], 0, data, sources, receivers)
        nrm = np.asarray(wall.normal)
        for c in (p.directivity_sources, p.directivity_receivers):
            for i in range(3):
                if nrm[i] > 1e-10:
                    assert (c.cartesian[:, i] > -1e-10).all()
                if nrm[i] < -1e-10:
                    assert (c.cartesian[:, i] < 1e-10).all()
        # the Euler-angle rotation equals the wall frame (data z -> normal, data x -> up)
        npt.assert_allclose(p.directivity_sources.cartesian,
                            ok.wall_frame_directions(sources.cartesian, wall.normal, wall.up_vector), atol=2e-15)
        npt.assert_allclose(p.directivity_receivers.cartesian,
                            ok.wall_frame_directions(receivers.cartesian, wall.normal, wall.up_vector), atol=2e-15)
        npt.assert_allclose(p.directivity_data.freq, np.abs(data.freq) * np.pi)
        npt.assert_array_equal(p.directivity_sources.weights, gold["ihta_source_weights"])


def ihta_data(gold, values=None):
    """The ihta file's directions and weights with data `values` (default: ones), as convert_sofa gives them."""
    shape = tuple(int(x) for x in gold["ihta_data_shape"])
    data = FrequencyData(np.ones(shape) if values is None else values, gold["ihta_N"])
    sources = sofa_pos(str(gold["ihta_source_type"]), gold["ihta_source_position"])
    receivers = sofa_pos(str(gold["ihta_receiver_type"]), gold["ihta_receiver_position"])
    sources.weights = gold["ihta_source_weights"]
    receivers.weights = gold["ihta_receiver_weights"]
    return data, sources, receivers


@pytest.mark.skipif(not SRC, reason="the reference's SOFA files are read when SPARROWPY_SRC is set")
def test_reader_against_stored_arrays(gold):
    from sparrowpy_gb300.sofa import convert_sofa, read_sofa
    for key, name in FILES.items():
        path = os.path.join(SRC, "tests", "test_data", name + ".sofa")
        with open(path, "rb") as fh:
            assert hashlib.sha256(fh.read()).hexdigest() == str(gold[f"{key}_sha256"])
        s = read_sofa(path)
        for v, shape, total in ast.literal_eval(str(gold[f"{key}_stats"])):
            a = getattr(s, v)
            assert list(a.shape) == shape and float(np.sum(a, dtype=np.float64)) == total, v
        npt.assert_array_equal(s.ReceiverPosition, gold[f"{key}_receiver_position"])
        if key != "ita_dodecahedron":
            data, src, rcv = convert_sofa(s)
            assert data.freq.shape == tuple(gold[f"{key}_data_shape"])
            assert src.csize == data.freq.shape[0] and rcv.csize == data.freq.shape[1]
    _known_answer(DirectivityMS(os.path.join(SRC, "tests", "test_data", "ITA_Dodecahedron.sofa")))


def test_coordinates_complex_frequency_data():
    f = FrequencyData(np.array([[1 + 2j, 3.0]]), [100, 200])
    assert f.freq.dtype == complex
    assert FrequencyData(np.array([1, 2]), [1, 2]).freq.dtype == float
    c = Coordinates.from_spherical_elevation(np.pi / 2, 0.0, 2.0)
    npt.assert_array_equal(c.cartesian, [[0.0, 2.0, 0.0]])
