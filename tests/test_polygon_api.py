"""Polygon and _Environment (sparrowpy/geometry.py:15-273), restating the reference's
tests/test_radiosity_geometry.py and the area formula of geometry.py:91-121."""
import numpy as np
import numpy.testing as npt
import pytest

import sparrowpy_gb300.geometry as geo
from sparrowpy_gb300.sound_object import Receiver, SoundSource

SQUARE = [[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]


def test_polygon_defaults_and_properties():
    poly = geo.Polygon(SQUARE, [0, 1, 0], [0, 0, 1])
    npt.assert_equal(poly.pts, np.array(SQUARE, float))
    npt.assert_almost_equal(poly.up_vector, [0, 1, 0])
    npt.assert_equal(poly.normal, [0, 0, 1])
    npt.assert_allclose(poly.center, [0.5, 0.5, 0])
    npt.assert_allclose(poly.size, [1, 1, 0])
    assert poly.n_points == 4
    assert poly.area == 1.0


def test_polygon_intersection():
    poly = geo.Polygon(SQUARE, [0, 1, 0], [0, 0, 1])
    npt.assert_allclose(poly.intersection([0.5, 0.5, 1], [0, 0, -1]), [0.5, 0.5, 0])
    assert poly.intersection([0.5, 0.5, 1], [0, 0, 1]) is None       # behind the ray
    assert poly.intersection([0.5, 0.5, 1], [1, 0, 0]) is None       # parallel
    assert poly.intersection([1.5, 0.5, 1], [0, 0, -1]) is None      # on the plane, outside the polygon
    npt.assert_allclose(poly.intersection([0.0, 0.0, 2], [0, 0, -1]), [0, 0, 0])  # a vertex


def test_polygon_on_surface():
    poly = geo.Polygon(SQUARE, [0, 1, 0], [0, 0, 1])
    assert poly.on_surface([0.25, 0.75, 0])
    assert poly.on_surface([1, 1, 0])
    assert not poly.on_surface([1.25, 0.5, 0])


@pytest.mark.parametrize("nv", [3, 5, 6, 8])
def test_polygon_area_of_regular_polygons(nv):
    a = 2 * np.pi * np.arange(nv) / nv
    pts = np.stack([np.cos(a), np.sin(a), np.zeros(nv)], axis=1)
    poly = geo.Polygon(pts, [1, 0, 0], [0, 0, 1])
    npt.assert_allclose(poly.area, 0.5 * nv * np.sin(2 * np.pi / nv), rtol=1e-14)
    npt.assert_allclose(poly.area, geo.calculate_area(pts[None])[0], rtol=1e-14)


def test_polygon_checks():
    with pytest.raises(AssertionError):
        geo.Polygon([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0.5]], [0, 1, 0], [0, 0, 1])  # not planar
    with pytest.raises(AssertionError):
        geo.Polygon(SQUARE, [0, 1, 0], [1, 0, 0])  # normal not perpendicular to the plane


def test_polygon_dict_round_trip():
    poly = geo.Polygon(SQUARE, [0, 1, 0], [0, 0, 1])
    d = poly.to_dict()
    npt.assert_array_equal(d['pts'], SQUARE)
    back = geo.Polygon.from_dict(d)
    npt.assert_array_equal(back.pts, poly.pts)
    npt.assert_array_equal(back.normal, poly.normal)


@pytest.mark.parametrize("c", [346.2, 346.18])
def test_environment(c):
    poly = geo.Polygon(SQUARE, [0, 1, 0], [0, 0, 1])
    source = SoundSource([0, 0, 0], [1, 0, 0], [0, 0, 1])
    receiver = Receiver([0, 0, 0], [1, 0, 0], [0, 0, 1])
    env = geo._Environment([poly], source, receiver, c)
    assert env.polygons == [poly] and env.speed_of_sound == c
    assert env.receiver is receiver and env.source is source
