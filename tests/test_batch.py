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
