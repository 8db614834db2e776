"""BRDF tables beyond one diffuse-plus-mirror material group, against the oracle.

* Per-patch scattering through the public API (set_wall_brdf per wall with
  create_from_scattering tables of different scattering), at 64 directions:
  every slot's normalised rows differ, so the (group, incoming direction)
  classes exceed 256 and the slot-wise exchange runs (a diffuse class and
  one class per mirror direction).
* A seeded random positive table (no diffuse-plus-mirror structure) on some
  walls, and tables of create_from_directional_scattering.

Tolerances: receiver histograms and E_total rel L2 <= 1e-4 (FP32) and
<= 1e-10 (FP64) against the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

SRC = np.array([2.0, 2.0, 1.5])
RCV = np.array([[3.0, 4.0, 1.5]])


def per_patch_scattering_room(precision, n_dirs=64, n_bins=2, seed=3, dims=(3.0, 2.0, 2.0), patch=1.0):
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import FrequencyData
    from sparrowpy_gb300.geometry import shoebox_room_stub
    from sparrowpy_gb300.radiosity import DirectionalRadiosityFast
    walls = scenes._patch_polygons(shoebox_room_stub(*dims), patch)
    r = DirectionalRadiosityFast.from_polygon(walls, patch, precision=precision)
    freqs = np.array([500.0, 1000.0])[:n_bins]
    dirs = hemisphere_directions(n_dirs)
    rng = np.random.default_rng(seed)
    for w in range(r.n_walls):
        tab = create_from_scattering(dirs, dirs, FrequencyData(rng.uniform(0.1, 0.9, n_bins), freqs),
                                     FrequencyData(rng.uniform(0.05, 0.3, n_bins), freqs))
        r.set_wall_brdf([w], tab, dirs, dirs)
    r.set_air_attenuation(FrequencyData(np.array([0.001, 0.002])[:n_bins], freqs))
    return r


def _solve(r, c=343.0, dt=1e-3, dur=0.1, k=8):
    from sparrowpy_gb300.coords import Coordinates
    r.bake_geometry()
    r.init_source_energy(Coordinates(*SRC))
    r.calculate_energy_exchange(c, dt, dur, k)
    mono = r.collect_energy_receiver_mono(Coordinates(RCV[:, 0], RCV[:, 1], RCV[:, 2])).time
    return mono, (c, dt, dur, k)


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp64", 1e-10)])
def test_per_patch_scattering_room_64_directions(precision, tol):
    from oracle.scene import scene_from_radiosity
    r = per_patch_scattering_room(precision)
    mono, (c, dt, dur, k) = _solve(r)
    assert r.exchange_stats["algorithm"] == "slotwise"
    ref = orc.solve(scene_from_radiosity(r), SRC, RCV, c, dt, dur, k)
    assert rel_l2(mono, ref["mono"]) < tol
    assert rel_l2(r._energy_exchange_etc, ref["etot"]) < tol


def random_table_room(precision, n_dirs, n_bins=2, seed=5):
    """Shoebox at 1 m patches: a seeded random positive BRDF table (no diffuse-plus-mirror structure) on the
    floor and ceiling, create_from_scattering tables on the other walls."""
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.brdf import hemisphere_directions
    from sparrowpy_gb300.coords import FrequencyData
    r = scenes.shoebox(1.0, n_dirs=n_dirs, n_bins=n_bins, scattering=0.4, absorption=0.15, seed=seed,
                       dims=(3.0, 2.0, 2.0), air_attenuation=[0.001, 0.002][:n_bins], precision=precision)
    rng = np.random.default_rng(seed)
    dirs = hemisphere_directions(n_dirs)
    tab = rng.uniform(0.05, 0.25, size=(n_dirs, n_dirs, n_bins)) / n_dirs * 8
    freqs = np.asarray(r._frequencies, float)
    r.set_wall_brdf([0, 1], FrequencyData(tab, freqs), dirs, dirs)
    return r


@pytest.mark.parametrize("n_dirs", [16, 64])
@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp64", 1e-10)])
def test_random_table_general_exchange(precision, tol, n_dirs):
    from oracle.scene import scene_from_radiosity
    r = random_table_room(precision, n_dirs)
    mono, (c, dt, dur, k) = _solve(r)
    assert r.exchange_stats["algorithm"] == "general"
    ref = orc.solve(scene_from_radiosity(r), SRC, RCV, c, dt, dur, k)
    assert rel_l2(mono, ref["mono"]) < tol
    assert rel_l2(r._energy_exchange_etc, ref["etot"]) < tol


def test_tensor_core_contraction_matches_cuda_cores():
    """The tcgen05 contraction (TF32 hi/lo split) against the CUDA-core one on the same solve: 64 directions,
    FP32; histograms within 1e-6 rel L2 of each other."""
    out = {}
    for tc in (True, False):
        r = random_table_room("fp32", 64)
        r.tensor_cores = tc
        out[tc] = _solve(r)[0]
        assert r.exchange_stats["algorithm"] == "general"
    assert rel_l2(out[True], out[False]) < 1e-6


@pytest.mark.parametrize("partial_sums", [True, False])
@pytest.mark.parametrize("room,algorithm", [("random", "general"), ("per_patch", "slotwise")])
@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp64", 1e-10)])
def test_long_histograms_general_and_slotwise(precision, tol, room, algorithm, partial_sums):
    """The benchmarked histogram shape (2200 bins: two full 1024-bin scatter windows and a partial third,
    17 contraction chunks of 128 bins with a partial last one) through the general (tensor cores at 64
    directions) and slot-wise exchanges, E_total as the last partial sum and order by order, 12 orders."""
    from oracle.scene import scene_from_radiosity
    r = random_table_room(precision, 64) if room == "random" else per_patch_scattering_room(precision, n_dirs=64)
    r.partial_sums = partial_sums
    mono, (c, dt, dur, k) = _solve(r, dt=5e-4, dur=1.1, k=12)
    st = r.exchange_stats
    assert st["algorithm"] == algorithm and st["partial_sums"] == partial_sums
    ref = orc.solve(scene_from_radiosity(r), SRC, RCV, c, dt, dur, k)
    assert rel_l2(mono, ref["mono"]) < tol
    assert rel_l2(r._energy_exchange_etc, ref["etot"]) < tol


@pytest.mark.parametrize("n_dirs", [16, 32])
@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp64", 1e-10)])
def test_directional_scattering_tables(precision, tol, n_dirs):
    """Floor and ceiling with create_from_directional_scattering tables (brdf.py:133-225): seeded random
    directional scattering coefficients normalised per incoming direction, absorption 0.2; the general
    exchange (tensor cores at 32 directions) against the oracle."""
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.brdf import create_from_directional_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import FrequencyData
    r = scenes.shoebox(1.0, n_dirs=n_dirs, n_bins=2, scattering=0.4, absorption=0.15, seed=9,
                       dims=(3.0, 2.0, 2.0), air_attenuation=[0.001, 0.002], precision=precision)
    freqs = np.asarray(r._frequencies, float)
    dirs = hemisphere_directions(n_dirs)
    sd = np.random.default_rng(9).random((n_dirs, n_dirs, 2))
    sd /= np.sum(sd, axis=1, keepdims=True)
    tab = create_from_directional_scattering(dirs, dirs, FrequencyData(sd, freqs),
                                             FrequencyData(np.full(2, 0.2), freqs))
    r.set_wall_brdf([0, 1], tab, dirs, dirs)
    mono, (c, dt, dur, k) = _solve(r)
    assert r.exchange_stats["algorithm"] == "general"
    ref = orc.solve(scene_from_radiosity(r), SRC, RCV, c, dt, dur, k)
    assert rel_l2(mono, ref["mono"]) < tol
    assert rel_l2(r._energy_exchange_etc, ref["etot"]) < tol
