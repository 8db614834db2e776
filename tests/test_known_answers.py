"""Known-answer tests of the path, restated from the reference's own tests.

* Diffuse shoebox against Kuttruff's reverberant-field decay (Eq. 4.7 and
  4.10), within 2 dB on bins 5..18 (sparrowpy tests/test_DRadiosityFast_order.py:49-117).
* ff_tilde equals the form factors for a diffuse BRDF without air
  attenuation, for perpendicular and parallel walls
  (tests/test_DRadiosityFast_order.py:11-46).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_order_vs_kuttruff(precision):
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    from sparrowpy_gb300.geometry import shoebox_room_stub
    X, Y, Z = 5.0, 3.0, 4.0
    c, dt, duration, K = 346.18, 1 / 500, 0.15, 3
    absorption = 0.1
    one = Coordinates(0, 0, 1, weights=1)
    freqs = np.array([500.0])
    brdf = create_from_scattering(one, one, FrequencyData([1.0], freqs), FrequencyData([absorption], freqs))
    walls = shoebox_room_stub(X, Y, Z)
    r = DirectionalRadiosityFast.from_polygon(walls, 1.0, precision=precision)
    r.set_wall_brdf(np.arange(len(walls)), brdf, one, one)
    r.set_air_attenuation(FrequencyData(np.zeros(1), freqs))
    r.bake_geometry()
    r.init_source_energy(Coordinates(2, 1.5, 2))
    r.calculate_energy_exchange(c, dt, duration, K, recalculate=True)
    etc = r.collect_energy_receiver_mono(Coordinates(3, 1.5, 2))
    S = 2 * (X * Y + X * Z + Y * Z)
    V = X * Y * Z
    A = S * absorption
    w0 = (4 / A) / V                      # Kuttruff Eq. 4.7
    t = etc.times
    analytic = w0 * np.exp(c * S * np.log(1 - A / S) / (4 * V) * (t - 0.03))  # Eq. 4.10
    with np.errstate(divide="ignore"):  # bins before the first arrival hold no energy
        model_db = 10 * np.log10(etc.time.reshape(-1))
    np.testing.assert_allclose(model_db[5:19], 10 * np.log10(analytic)[5:19], atol=2)


def _two_walls(kind):
    from sparrowpy_gb300.geometry import Polygon
    floor = Polygon([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], [1, 0, 0], [0, 0, 1])
    if kind == "perpendicular":
        other = Polygon([[0, 0, 0], [0, 1, 0], [0, 1, 1], [0, 0, 1]], [0, 0, 1], [1, 0, 0])
    else:
        other = Polygon([[0, 0, 1], [0, 1, 1], [1, 1, 1], [1, 0, 1]], [1, 0, 0], [0, 0, -1])
    return [floor, other]


@pytest.mark.parametrize("kind", ["perpendicular", "parallel"])
def test_form_factors_tilde_equal_form_factors_for_diffuse(kind):
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import hemisphere_directions
    from sparrowpy_gb300.coords import FrequencyData
    walls = _two_walls(kind)
    r = DirectionalRadiosityFast.from_polygon(walls, 0.5, precision="fp64")
    dirs = hemisphere_directions(4)
    freqs = np.array([250.0, 500.0, 1000.0, 2000.0])
    diffuse = FrequencyData(np.full((4, 4, 4), 1 / np.pi), freqs)  # Lambertian, stored x pi = 1
    r.set_wall_brdf(np.arange(2), diffuse, dirs, dirs)
    r.set_air_attenuation(FrequencyData(np.zeros(4), freqs))
    r.bake_geometry()
    fft = r._form_factors_tilde
    ff = r._form_factors
    assert fft.shape == (8, 8, 4, 4)
    for i in range(8):
        for j in range(8):
            expect = ff[i, j] if i < j else ff[j, i]
            np.testing.assert_allclose(fft[i, j], expect, rtol=1e-12, atol=1e-15)
