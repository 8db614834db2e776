"""State files (RadiosityFast.py:828-839): write, from_read, and resume without a bake.

The reference restores the visibility matrix and form factors from the file
and runs the exchange without bake_geometry(); here the device pair data is
rebuilt from them.  The check is bit-identical: collecting from the restored
histograms, and a new exchange after from_read, both give the original
receiver histograms exactly.

Files in the layout the reference's write() produces (pyfar.io.write of
to_dict(): nested lists for arrays, the BRDF tables as ndarray members,
the per-wall direction sets as Coordinates objects) are made here by a
restatement of pyfar's codec (no pyfar is installed, and the reference's
test data holds no such file, so this layout is not pinned to pyfar's own
output); from_read must restore the same object from them.
"""
import io
import json
import zipfile

import numpy as np
import pytest

from conftest import acoustics, load_golden, radiosity_from_golden


def _pyfar_style_write(path, values):
    """pyfar.io.write(path, **values) for builtins, lists, ndarrays and Coordinates (the codec's type hints)."""
    from sparrowpy_gb300.coords import _cart, is_coordinates
    members = {}

    def npy(a, where):
        buf = io.BytesIO()
        np.save(buf, np.asarray(a), allow_pickle=False)
        members[where] = buf.getvalue()
        return ["$ndarray", where]

    def enc(obj, where):
        if isinstance(obj, np.ndarray):
            return npy(obj, where)
        if is_coordinates(obj):
            w = obj.weights
            return ["$Coordinates", {"_data": npy(_cart(obj), f"{where}/_data"),
                                     "_weights": None if w is None else npy(w, f"{where}/_weights"),
                                     "_comment": ""}]
        if isinstance(obj, (list, tuple)):
            return [enc(v, f"{where}/{i}") for i, v in enumerate(obj)]
        if isinstance(obj, dict):
            return {k: enc(v, f"{where}/{k}") for k, v in obj.items()}
        if isinstance(obj, np.generic):
            return [f"${type(obj).__name__}", obj.item()]
        return obj

    wrapped = {k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in values.items()}  # to_dict
    wrapped["pyfar.__version__"] = "0.6.5"
    members["builtin_wrapper/$BuiltinsWrapper"] = json.dumps(enc(wrapped, "builtin_wrapper")).encode()
    with zipfile.ZipFile(path, "w", compression=zipfile.ZIP_DEFLATED) as z:
        for m, b in members.items():
            z.writestr(m, b)


def _small_room():
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import FrequencyData
    from sparrowpy_gb300.geometry import shoebox_room_stub
    r = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(2, 1.5, 1), 0.5)
    dirs = hemisphere_directions(8)
    f = np.array([500.0, 1000.0])
    r.set_wall_brdf(np.arange(3), create_from_scattering(dirs, dirs, FrequencyData([0.3, 0.5], f),
                                                         FrequencyData([0.1, 0.2], f)), dirs, dirs)
    r.set_wall_brdf(np.arange(3, 6), create_from_scattering(dirs, dirs, FrequencyData([0.6, 0.7], f),
                                                            FrequencyData([0.05, 0.1], f)), dirs, dirs)
    r.set_air_attenuation(FrequencyData([0.001, 0.002], f))
    return r


def test_reads_the_reference_file_layout(tmp_path):
    """A to_dict() written in pyfar's layout reads back as the same inputs (no GPU needed)."""
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.coords import _cart
    r = _small_room()
    values = dict(r.to_dict())
    values["brdf_incoming_directions"] = list(r._brdf_incoming_directions)  # to_dict's tolist of the object arrays
    values["brdf_outgoing_directions"] = list(r._brdf_outgoing_directions)
    _pyfar_style_write(tmp_path / "ref.far", values)
    r2 = DirectionalRadiosityFast.from_read(tmp_path / "ref.far")
    np.testing.assert_array_equal(r2._patches_points, r._patches_points)
    np.testing.assert_array_equal(r2._brdf_index, r._brdf_index)
    assert len(r2._brdf) == len(r._brdf) and all(np.array_equal(a, b) for a, b in zip(r2._brdf, r._brdf))
    assert r2._brdf_incoming_directions.shape == (6,)
    for a, b in zip(r2._brdf_incoming_directions, r._brdf_incoming_directions):
        np.testing.assert_array_equal(_cart(a), _cart(b))
        np.testing.assert_array_equal(a.weights, b.weights)
    np.testing.assert_array_equal(r2._air_attenuation, r._air_attenuation)
    np.testing.assert_array_equal(r2._frequencies, r._frequencies)


def test_unknown_pyfar_types_are_refused(tmp_path):
    from sparrowpy_gb300 import far
    with zipfile.ZipFile(tmp_path / "sig.far", "w") as z:
        z.writestr("signal/$Signal", json.dumps({"_data": ["$ndarray", "signal/_data"]}))
    with pytest.raises(NotImplementedError, match="Signal"):
        far.read(tmp_path / "sig.far")


@pytest.mark.gpu
def test_reference_layout_file_solves_like_the_original(tmp_path):
    """From the pyfar-layout file: the same receiver histograms as the object it was written from."""
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.coords import Coordinates
    r = _small_room()
    src, rcv = Coordinates(0.5, 0.6, 0.4), Coordinates(1.4, 0.9, 0.6)
    r.bake_geometry()
    r.init_source_energy(src)
    r.calculate_energy_exchange(343.0, 1e-3, 0.05, 5)
    mono = r.collect_energy_receiver_mono(rcv).time
    values = dict(r.to_dict())
    values["brdf_incoming_directions"] = list(r._brdf_incoming_directions)
    values["brdf_outgoing_directions"] = list(r._brdf_outgoing_directions)
    _pyfar_style_write(tmp_path / "ref.far", values)
    r2 = DirectionalRadiosityFast.from_read(tmp_path / "ref.far")
    np.testing.assert_array_equal(r2.collect_energy_receiver_mono(rcv).time, mono)
    r2.init_source_energy(src)
    r2.calculate_energy_exchange(343.0, 1e-3, 0.05, 5, recalculate=True)  # no bake_geometry()
    np.testing.assert_array_equal(r2.collect_energy_receiver_mono(rcv).time, mono)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["shoebox_126", "rot"])
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


def test_kang_objects_read_from_the_reference_layout(tmp_path):
    """RadiosityKang / DirectionalRadiosityKang.from_read on a file in the reference's layout
    (pyfar.io.write(**to_dict()): the walls as a list of dicts), written by the restated encoder; walls not
    yet run (no energy matrices), so no device work."""
    from sparrowpy_gb300.coords import Coordinates, FrequencyData
    from sparrowpy_gb300.geometry import shoebox_room_stub
    from sparrowpy_gb300.kang import DirectionalRadiosityKang, PatchesDirectionalKang, RadiosityKang
    walls = shoebox_room_stub(2, 1.5, 1)
    radi = RadiosityKang(walls, 0.5, 2, 0.1, speed_of_sound=343.0, sampling_rate=1000)
    d = radi.to_dict()
    path = tmp_path / "kang.far"
    _pyfar_style_write(path, d)
    back = RadiosityKang.from_read(path)
    assert (back.patch_size, back.max_order_k, back.ir_length_s) == (0.5, 2, 0.1)
    for a, b in zip(radi.patch_list, back.patch_list, strict=True):
        np.testing.assert_array_equal(a.pts, b.pts)
        assert a.wall_id == b.wall_id and b.E_matrix is None
        np.testing.assert_array_equal(a.other_wall_ids, b.other_wall_ids)
    g = np.linspace(0.1, 1.0, 6)
    dirs = Coordinates.from_cartesian(np.stack([np.sin(g), np.zeros(6), np.cos(g)], 1), weights=np.full(6, 1 / 6))
    data = FrequencyData(np.random.default_rng(1).uniform(0, 1, (6, 6, 2)), [500.0, 1000.0])
    dwalls = [PatchesDirectionalKang(w, 0.5, [j for j in range(6) if j != i], i, data, dirs, dirs)
              for i, w in enumerate(walls)]
    drad = DirectionalRadiosityKang(dwalls, 0.5, 2, 0.1, None, speed_of_sound=343.0)
    _pyfar_style_write(tmp_path / "dkang.far", drad.to_dict())
    dback = DirectionalRadiosityKang.from_read(tmp_path / "dkang.far")
    for a, b in zip(drad.patch_list, dback.patch_list, strict=True):
        np.testing.assert_array_equal(a.directivity_data.freq, b.directivity_data.freq)
        assert a.directivity_sources == b.directivity_sources
