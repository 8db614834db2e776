"""BRDF constructors (sparrowpy/brdf.py:8-225), restating the reference's tests/test_brdf.py
checks on the returned tables: energy conservation (the cosine-weighted integral over the
outgoing directions is 1 - absorption, 1 decimal as the reference) and reciprocity."""
import numpy as np
import numpy.testing as npt
import pytest

from sparrowpy_gb300.brdf import create_from_directional_scattering, create_from_scattering, sph_gaussian
from sparrowpy_gb300.coords import FrequencyData

FREQS = [100, 200, 400]


def upper(sh_order):
    coords = sph_gaussian(sh_order=sh_order)
    return coords[coords.z > 0]


def check_energy_conservation(receivers, receiver_weights, data, absorption_data=0):
    w = np.array(receiver_weights, dtype=float)
    w *= 2 * np.pi / np.sum(w)
    w *= np.cos(receivers.colatitude)
    energy = np.sum(np.asarray(data.freq) * w[..., np.newaxis], axis=1)
    npt.assert_almost_equal(energy, 1 - absorption_data, decimal=1)


def check_reciprocity(data):
    a = np.asarray(data.freq)
    npt.assert_almost_equal(a, np.swapaxes(a, 0, 1))


@pytest.mark.parametrize('scattering_data', [0, 0.3, 1])
@pytest.mark.parametrize('absorption_data', [0, 0.3, 1])
@pytest.mark.parametrize('sh_order', [5, 11])
def test_create_from_scattering_energy_and_reciprocity(scattering_data, absorption_data, sh_order):
    coords = upper(sh_order)
    brdf = create_from_scattering(coords, coords, FrequencyData(scattering_data + np.zeros(3), FREQS),
                                  FrequencyData(absorption_data + np.zeros(3), FREQS))
    check_energy_conservation(coords, coords.weights, brdf, absorption_data)
    check_reciprocity(brdf)


@pytest.mark.parametrize('absorption_data', [0, 0.5])
@pytest.mark.parametrize('sh_order', [5, 11])
def test_directional_specular(absorption_data, sh_order):
    coords = upper(sh_order)
    data = np.zeros((coords.csize, coords.csize, 3))
    data[np.arange(coords.csize), np.arange(coords.csize)] = 1
    brdf = create_from_directional_scattering(coords, coords, FrequencyData(data, FREQS),
                                              FrequencyData(absorption_data + np.zeros(3), FREQS))
    check_energy_conservation(coords, coords.weights, brdf, absorption_data)
    check_reciprocity(brdf)


@pytest.mark.parametrize('absorption_data', [0, 0.3, 1])
@pytest.mark.parametrize('sh_order', [7, 11])
def test_directional_diffuse(absorption_data, sh_order):
    coords = upper(sh_order)
    coords.weights = coords.weights * 2 * np.pi / np.sum(coords.weights)
    data = np.cos(coords.colatitude)[None, :, None] * coords.weights[None, :, None] / np.pi * \
        np.ones((coords.csize, coords.csize, 3))
    npt.assert_almost_equal(np.sum(data, axis=1), 1, decimal=2)
    brdf = create_from_directional_scattering(coords, coords, FrequencyData(data, FREQS),
                                              FrequencyData(absorption_data + np.zeros(3), FREQS))
    check_energy_conservation(coords, coords.weights, brdf, absorption_data)
    check_reciprocity(brdf)
    npt.assert_almost_equal(brdf.freq, (1 - absorption_data) / np.pi, decimal=2)


@pytest.mark.parametrize('absorption_data', [0, 0.5])
@pytest.mark.parametrize('sh_order', [5, 11])
def test_directional_two_directions(absorption_data, sh_order):
    coords = upper(sh_order)
    data = np.zeros((coords.csize, coords.csize, 3))
    data[np.arange(coords.csize), np.arange(coords.csize)] = 0.5
    refl = coords.copy()
    refl.azimuth = refl.azimuth + np.pi
    idx = coords.find_nearest(refl)[0][0]
    data[np.arange(coords.csize), idx] += 0.5
    npt.assert_array_equal(np.sum(data, axis=1), 1)
    brdf = create_from_directional_scattering(coords, coords, FrequencyData(data, FREQS),
                                              FrequencyData(absorption_data + np.zeros(3), FREQS))
    check_energy_conservation(coords, coords.weights, brdf, absorption_data)
    check_reciprocity(brdf)


@pytest.mark.parametrize('absorption_data', [0, 0.5])
@pytest.mark.parametrize('sh_order', [5, 11])
def test_directional_random(absorption_data, sh_order):
    coords = upper(sh_order)
    rng = np.random.default_rng(1337)
    data = rng.random((coords.csize, coords.csize, 3))
    data /= np.sum(data, axis=1, keepdims=True)
    brdf = create_from_directional_scattering(coords, coords, FrequencyData(data, FREQS),
                                              FrequencyData(absorption_data + np.zeros(3), FREQS))
    check_energy_conservation(coords, coords.weights, brdf, absorption_data)


def test_directional_input_errors():
    coords = upper(3)
    good = FrequencyData(np.ones((coords.csize, coords.csize, 1)), [100])
    with pytest.raises(TypeError):
        create_from_directional_scattering(np.zeros((3, 3)), coords, good)
    with pytest.raises(TypeError):
        create_from_directional_scattering(coords, coords, FrequencyData(np.ones((2, 2, 1)), [100]))
    with pytest.raises(NotImplementedError):
        create_from_directional_scattering(coords, coords, good, file_path="brdf.sofa")
    with pytest.raises(NotImplementedError):
        create_from_scattering(coords, coords, FrequencyData([0.5], [100]), file_path="brdf.sofa")
