"""Pin the FP64 CPU oracle to golden vectors produced by the sparrowpy reference.

The fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py)
hold the reference's own outputs for four scenes: a 1 m cube at 0.5 m
patches, the 5 x 6 x 3 m shoebox at 1 m (126 patches) and a rotated room with
an occluder in generic position.
"""
import numpy as np
import pytest

from conftest import acoustics, load_golden, rel_l2, scene_from_golden
from oracle import oracle as orc

SCENES = ["cube", "shoebox_126", "rot", "tri"]


@pytest.fixture(scope="module", params=SCENES)
def solved(request):
    g = load_golden(request.param)
    sc = scene_from_golden(g)
    c, dt, duration, k = acoustics(g)
    bk = orc.bake(sc)
    e0dir, d0, svis = orc.init_source(sc, bk, g["source"])
    nt = int(duration / dt)
    etot = orc.exchange(sc, bk, e0dir, d0, c, dt, nt, k)
    return g, sc, bk, e0dir, d0, svis, etot


def test_centers_areas(solved):
    g, sc, bk, *_ = solved
    np.testing.assert_array_equal(bk["centers"], g["centers"])
    np.testing.assert_allclose(bk["areas"], g["areas"], rtol=1e-14)


def test_visibility_exact(solved):
    g, sc, bk, *_ = solved
    np.testing.assert_array_equal(bk["vis"], g["V"])
    np.testing.assert_array_equal(bk["pairs"], g["visible_patches"])


def test_form_factors(solved):
    g, sc, bk, *_ = solved
    np.testing.assert_allclose(bk["ff"], g["ff_pairs"], rtol=1e-11, atol=0)


def test_outgoing_index_map(solved):
    g, sc, bk, *_ = solved
    np.testing.assert_array_equal(bk["p2o_dense"], g["p2o"].astype(np.int64))


def test_form_factors_tilde(solved):
    g, sc, bk, *_ = solved
    fft = orc.form_factors_tilde(sc, bk)
    if "ff_tilde" in g:
        np.testing.assert_allclose(fft, g["ff_tilde"], rtol=1e-11, atol=1e-300)
    else:
        sel = g["ff_tilde_pairs"]
        np.testing.assert_allclose(fft[sel[:, 0], sel[:, 1]], g["ff_tilde_sel"][0], rtol=1e-11)
        np.testing.assert_allclose(fft[sel[:, 1], sel[:, 0]], g["ff_tilde_sel"][1], rtol=1e-11)


def test_source_energy(solved):
    g, sc, bk, e0dir, d0, svis, etot = solved
    np.testing.assert_array_equal(svis, g["svis"])
    np.testing.assert_allclose(d0, g["d0"], rtol=1e-15)
    np.testing.assert_allclose(e0dir, g["e0dir"], rtol=1e-12, atol=0)


def test_energy_exchange(solved):
    g, sc, bk, e0dir, d0, svis, etot = solved
    if "etot" in g:
        np.testing.assert_allclose(etot, g["etot"], rtol=1e-10, atol=1e-300)
    else:
        np.testing.assert_allclose(etot[g["etot_rows_index"]], g["etot_rows"], rtol=1e-10, atol=1e-300)
        np.testing.assert_allclose(etot.sum(axis=-1), g["etot_time_sum"], rtol=1e-10, atol=1e-300)


def test_collect(solved):
    g, sc, bk, e0dir, d0, svis, etot = solved
    c, dt, duration, k = acoustics(g)
    mono = orc.collect(sc, bk, etot, g["receivers"], c, dt)
    assert rel_l2(mono, g["mono"]) < 1e-12
    if "patchwise" in g:
        pw = orc.collect(sc, bk, etot, g["receivers"], c, dt, patchwise=True)
        np.testing.assert_allclose(pw, g["patchwise"], rtol=1e-10, atol=1e-300)
