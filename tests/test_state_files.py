"""State files on the GPU (RadiosityFast.py:828-839): write, from_read, and resume without a bake.

The reference restores the visibility matrix and form factors from the file
and runs the exchange without bake_geometry(); here the device pair data is
rebuilt from them.  The check is bit-identical: collecting from the restored
histograms, and a new exchange after from_read, both give the original
receiver histograms exactly.
"""
import numpy as np
import pytest

from conftest import acoustics, load_golden, radiosity_from_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cfg1", "rot"])
def test_resume_from_state_file_without_bake(name, tmp_path):
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.coords import Coordinates
    g = load_golden(name)
    c, dt, duration, k = acoustics(g)
    rcv = np.atleast_2d(g["receivers"])
    receivers = Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])
    r = radiosity_from_golden(g, "fp32")
    r.bake_geometry()
    r.init_source_energy(Coordinates(*g["source"]))
    r.calculate_energy_exchange(c, dt, duration, k)
    mono = r.collect_energy_receiver_mono(receivers).time
    r.write(tmp_path / "state.far")

    r2 = DirectionalRadiosityFast.from_read(tmp_path / "state.far")
    assert r2 == r
    np.testing.assert_array_equal(r2.collect_energy_receiver_mono(receivers).time, mono)

    r3 = DirectionalRadiosityFast.from_read(tmp_path / "state.far")
    r3.init_source_energy(Coordinates(*g["source"]))
    r3.calculate_energy_exchange(c, dt, duration, k, recalculate=True)  # no bake_geometry()
    np.testing.assert_array_equal(r3.collect_energy_receiver_mono(receivers).time, mono)
    np.testing.assert_array_equal(r3._visibility_matrix, g["V"])
