"""Batched rooms (seeded shoeboxes, solved one after another): each room's receiver histograms against the oracle.

Tolerance: rel L2 <= 1e-4 (FP32 exchange).
"""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_rooms_match_oracle():
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300.batch import build_room, shoebox_rooms, solve_rooms
    rooms = shoebox_rooms(3, seed=11, patch_size=0.5, dims_range=(1.5, 3.0), n_dirs=8, n_bins=2, n_receivers=2)
    monos, ms, patches = solve_rooms(rooms, etc_duration=0.05, max_reflection_order=5)
    assert len(monos) == 3 and all(m > 0 for m in ms)
    for room, mono, n in zip(rooms, monos, patches):
        r = build_room(room, "fp64")
        assert r.n_patches == n
        ref = orc.solve(scene_from_radiosity(r), room["source"], room["receivers"], 343.0, 1e-3, 0.05, 5)
        assert rel_l2(mono, ref["mono"]) < 1e-4


def _rooms(n=3, seed=11):
    from sparrowpy_gb300.batch import shoebox_rooms
    return shoebox_rooms(n, seed=seed, patch_size=0.5, dims_range=(1.5, 3.0), n_dirs=8, n_bins=2, n_receivers=2)


@pytest.mark.parametrize("partial_sums", [True, False])
def test_persistent_batch_matches_rooms_one_by_one(partial_sums):
    """All orders of three rooms in one persistent launch, for every tile choice the tuner can pick (and its
    room-after-room alternative on the prepared plans), with E_total as the last partial sum and order by
    order: the same receiver histograms as the rooms solved one after another in the same form
    (rel L2 <= 1e-6), and the oracle's (1e-4)."""
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300.batch import BatchTuner, build_room, solve_rooms, solve_rooms_batched
    rooms = _rooms()
    ref, _, _ = solve_rooms(rooms, etc_duration=0.06, max_reflection_order=6, partial_sums=partial_sums)
    for choice in BatchTuner.CANDIDATES:
        got, stats = solve_rooms_batched(rooms, etc_duration=0.06, max_reflection_order=6, force_choice=choice,
                                         partial_sums=partial_sums)
        assert stats["waves"][0]["rooms"] == 3
        for a, b in zip(got, ref):
            assert rel_l2(a, b) < 1e-6, choice
    for room, mono in zip(rooms, got):
        r = build_room(room, "fp64")
        orc_ref = orc.solve(scene_from_radiosity(r), room["source"], room["receivers"], 343.0, 1e-3, 0.06, 6)
        assert rel_l2(mono, orc_ref["mono"]) < 1e-4


def test_persistent_batch_tuner_keeps_its_choice():
    from sparrowpy_gb300.batch import BatchTuner, solve_rooms_batched
    tuner = BatchTuner(probe_orders=2)
    _, stats = solve_rooms_batched(_rooms(2), etc_duration=0.06, max_reflection_order=6, tuner=tuner)
    (key, times), = tuner.timings.items()
    assert set(times) == set(BatchTuner.CANDIDATES) and all(t > 0 for t in times.values())
    w = stats["waves"][0]
    assert (w["window_bins"], w["ctas_per_sm"]) == min(times, key=times.get)
    _, stats2 = solve_rooms_batched(_rooms(2, seed=12), etc_duration=0.06, max_reflection_order=6, tuner=tuner)
    assert len(tuner.timings) == 1 or stats2["waves"][0]["window_bins"] in (512, 1024)


def test_persistent_batch_bounded_wait_reports_timeout():
    """A dependency wait that cannot be met (the test hook: a count nothing reaches) gives up after its poll limit,
    the call returns SP_ERR_TIMEOUT, and the next launch on the same device succeeds."""
    from sparrowpy_gb300 import _native as nat
    from sparrowpy_gb300.batch import PreparedWave, solve_rooms
    rooms = _rooms(2)
    pw = PreparedWave(rooms, 343.0, 1e-3, 60, 6)
    rc, _, _ = pw.launch((512, 1), wait_limit=2000, force_timeout=True)
    assert rc == nat.SP_ERR_TIMEOUT
    rc, _, items = pw.launch((512, 1))
    assert rc == nat.SP_OK and items > 0
    ref, _, _ = solve_rooms(rooms, etc_duration=0.06, max_reflection_order=6)
    for a, b in zip(pw.results(rooms), ref):
        assert rel_l2(a, b) < 1e-6


def test_batch_of_mixed_shapes_runs_room_by_room():
    """Rooms of different direction counts in one wave, and a histogram length that is not a multiple of 4:
    the persistent launch does not take them, so the wave runs the rooms' own launches; the histograms equal
    the rooms solved one after another (rel L2 <= 1e-6)."""
    from sparrowpy_gb300.batch import BatchTuner, shoebox_rooms, solve_rooms, solve_rooms_batched
    rooms = _rooms(2) + shoebox_rooms(1, seed=5, patch_size=0.5, dims_range=(1.5, 3.0), n_dirs=16, n_bins=2,
                                      n_receivers=2)
    for dur, sub in ((0.06, rooms), (0.061, rooms[:2])):
        ref, _, _ = solve_rooms(sub, etc_duration=dur, max_reflection_order=5)
        tuner = BatchTuner()
        got, stats = solve_rooms_batched(sub, etc_duration=dur, max_reflection_order=5, tuner=tuner)
        assert [w["mode"] for w in stats["waves"]] == ["rooms"] and not tuner.timings
        for a, b in zip(got, ref):
            assert rel_l2(a, b) < 1e-6
