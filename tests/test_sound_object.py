"""Sound objects and source directivity (sparrowpy/sound_object.py; tests/test_radiosity_sound_object.py).

The CPU tests restate the reference's sound-object tests: construction and
normalisation, errors, defaults, and the azimuth/elevation convention of
_get_metrics, whose known answer is exact; the directivity read from the
reference's SOFA file and its known answer are in test_sofa.py.
The GPU test checks the directivity path of init_source_energy
(RadiosityFast.py:500-519): E0dir of a directive source equals the
omnidirectional E0dir times the directivity towards each patch centre,
band by band.
"""
import numpy as np
import numpy.testing as npt
import pytest

import sparrowpy_gb300.sound_object as so


@pytest.mark.parametrize("cls", [so.SoundObject, so.SoundSource, so.Receiver])
def test_sound_object(cls):
    o = cls([0, 0, 0], [2, 0, 0], [0, 0, 2])
    npt.assert_equal(o.position, np.array([0, 0, 0]))
    npt.assert_equal(o.view, np.array([1, 0, 0]))
    npt.assert_equal(o.up, np.array([0, 0, 1]))


@pytest.mark.parametrize("cls", [so.SoundObject, so.SoundSource, so.Receiver])
@pytest.mark.parametrize(("position", "view", "up"), [
    ("a", [1, 0, 0], [0, 0, 1]),
    ([0, 0, 0], [1, 0, 0], 1),
    ([0, 0, 0], ["a"], [0, 0, 1]),
])
def test_sound_object_error(cls, position, view, up):
    with pytest.raises((ValueError, AssertionError)):
        cls(position, view, up)


def test_sound_source_defaults_and_errors():
    s = so.SoundSource([0, 0, 0], [2, 0, 0], [0, 0, 2])
    assert s.sound_power == 1 and s.directivity is None
    with pytest.raises((ValueError, AssertionError)):
        so.SoundSource([0, 0, 0], [2, 0, 0], [0, 0, 2], "a", 1)
    with pytest.raises((ValueError, AssertionError)):
        so.SoundSource([0, 0, 0], [2, 0, 0], [0, 0, 2], None, "a")
    with pytest.raises(FileNotFoundError):
        so.DirectivityMS("directivity.sofa")
    with pytest.raises(ValueError):
        so.DirectivityMS()


def test_get_metrics_known_answer():
    az, el = so._get_metrics([0, 0, 2], [-0.707106781186548, 0, 0.707106781186548], [0, 1, 0], [-1, 0, -2])
    assert az == -120.96375653207352
    assert el == 0


def test_nearest_direction_lookup():
    """The value of the sampled direction nearest to the target, in the source's frame."""
    from sparrowpy_gb300.coords import Coordinates
    # samples on the frame axes: (az, el) = (0, 0) is the view direction -z' = view
    az = np.deg2rad([0.0, 90.0, 180.0, -90.0, 0.0])
    el = np.deg2rad([0.0, 0.0, 0.0, 0.0, 90.0])
    dirs = Coordinates.from_spherical_colatitude(az, np.pi / 2 - el, 1)
    data = np.array([[1.0, 10.0], [2.0, 20.0], [3.0, 30.0], [4.0, 40.0], [5.0, 50.0]])
    d = so.DirectivityMS.from_arrays(data, [500.0, 1000.0], dirs)
    src = so.SoundSource([0, 0, 0], [1, 0, 0], [0, 0, 1], directivity=d)
    # the source frame: z' = -view = -x, y' = up = z, x' = view x up = -y
    targets = np.array([[-5.0, 0, 0], [0, 5.0, 0], [5.0, 0, 0], [0, -5.0, 0], [0, 0, 5.0]])
    az_t, el_t = so._get_metrics(src.position, src.view, src.up, targets)
    npt.assert_allclose(el_t, [0, 0, 0, 0, 90], atol=1e-12)
    npt.assert_allclose(np.abs(az_t[:4]), [180, 90, 0, 90], atol=1e-12)
    got = src.get_directivity(targets, 990.0)                 # the 1000 Hz bin
    # -x is -z' (behind: azimuth 180), +y is -x' (azimuth 90), +x is the view
    # (azimuth 0), -y is azimuth -90 and +z is the pole of the frame
    npt.assert_array_equal(got, [30.0, 20.0, 10.0, 40.0, 50.0])


@pytest.mark.gpu
def test_directive_source_energy():
    import torch
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    from sparrowpy_gb300.geometry import shoebox_room_stub
    f = np.array([500.0, 1000.0])
    dirs = hemisphere_directions(8)
    rng = np.random.default_rng(4)
    grid = Coordinates.from_cartesian(rng.standard_normal((200, 3)) / 1.0)
    grid = Coordinates.from_cartesian(grid.cartesian / np.linalg.norm(grid.cartesian, axis=1, keepdims=True))
    data = rng.uniform(0.2, 2.0, size=(200, 2))
    directivity = so.DirectivityMS.from_arrays(data, f, grid)
    src_pos = [1.2, 0.9, 0.7]
    src = so.SoundSource(src_pos, [1, 0.3, 0], [0, 0, 1], directivity=directivity)

    def room():
        r = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(3, 2, 2), 0.5, precision="fp64")
        r.set_wall_brdf(np.arange(6), create_from_scattering(dirs, dirs, FrequencyData([0.3, 0.5], f),
                                                             FrequencyData([0.1, 0.2], f)), dirs, dirs)
        r.set_air_attenuation(FrequencyData([0.001, 0.002], f))
        return r

    omni = room()
    omni.init_source_energy(Coordinates(*src_pos))
    directive = room()
    directive.init_source_energy(src)
    fac = np.stack([np.real(src.get_directivity(omni.patches_center, fb)) for fb in f], axis=-1)  # (N, B)
    e_omni = omni._energy_init_source
    e_dir = directive._energy_init_source
    assert np.any(e_omni > 0)
    npt.assert_allclose(e_dir, e_omni * fac[:, None, :], rtol=1e-14, atol=0)
    torch.cuda.synchronize()
