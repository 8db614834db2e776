"""The HDF5 reader on the format's earliest layout (sparrowpy_gb300/hdf5.py).

The reference's SOFA fixtures (test_sofa.py) use version-2 object headers
and dense groups.  Many SOFA files, e.g. those of older HDF5 releases, use a
version-0 superblock, version-1 object headers and a symbol-table group.
tests/hdf5_earliest.py writes that layout from the published format
specification; the reader must give back the arrays, attributes and the
SOFA view of the file: contiguous, compact and chunked data (2 x 3 chunks
with padded edge chunks, with and without shuffle + deflate), float64 and
int32, fixed-length and variable-length string attributes.
"""
import numpy as np
import numpy.testing as npt

from hdf5_earliest import Writer
from sparrowpy_gb300 import hdf5
from sparrowpy_gb300.sofa import convert_sofa, read_sofa


def _sofa_like(path, rng):
    w = Writer()
    data = rng.uniform(0, 1, (5, 7, 3))
    rpos = rng.normal(size=(7, 3))
    spos = np.stack([rng.uniform(0, 360, 5), rng.uniform(0, 90, 5), np.ones(5)], axis=1)
    links = {
        "Data.Real": w.dataset(data, "chunked", chunks=(2, 3, 3), filters=True),
        "Data.Imag": w.dataset(np.zeros_like(data), "chunked", chunks=(2, 3, 3)),
        "N": w.dataset(np.array([125.0, 250.0, 500.0]), "compact", attrs={"Units": "hertz"}),
        "ReceiverPosition": w.dataset(rpos, attrs={"Type": "cartesian", "Units": "vl:metre"}),
        "SourcePosition": w.dataset(spos, attrs={"Type": "vl:spherical", "Units": "degree, degree, metre"}),
        "SourceWeights": w.dataset(np.full(5, 0.2)),
        "ReceiverWeights": w.dataset(np.full(7, 1 / 7)),
        "Counts": w.dataset(np.arange(12, dtype=np.int32).reshape(3, 4), "chunked", chunks=(2, 3)),
        "M": w.dataset(np.zeros(5), attrs={"NAME": "This is a netCDF dimension but not a netCDF variable.     5"}),
    }
    w.finish(path, links, root_attrs={"Conventions": "SOFA", "DataType": "vl:TF", "Version": [2.1]})
    return data, rpos, spos


def test_earliest_layout_datasets_and_attributes(tmp_path):
    rng = np.random.default_rng(4)
    path = tmp_path / "old.sofa"
    data, rpos, spos = _sofa_like(path, rng)
    f = hdf5.File(path)
    assert f.attrs["Conventions"].value() == "SOFA"
    assert f.attrs["DataType"].value() == "TF"
    npt.assert_array_equal(f.attrs["Version"].value(), [2.1])
    ds = f.datasets()
    npt.assert_array_equal(ds["Data.Real"].read(), data)
    npt.assert_array_equal(ds["Data.Imag"].read(), np.zeros_like(data))
    npt.assert_array_equal(ds["N"].read(), [125.0, 250.0, 500.0])
    npt.assert_array_equal(ds["Counts"].read(), np.arange(12).reshape(3, 4))
    assert ds["Counts"].read().dtype == np.int32
    npt.assert_array_equal(ds["ReceiverPosition"].read(), rpos)
    assert ds["ReceiverPosition"].attrs["Units"].value() == "metre"
    assert ds["SourcePosition"].attrs["Type"].value() == "spherical"


def test_earliest_layout_as_sofa(tmp_path):
    rng = np.random.default_rng(5)
    path = tmp_path / "old.sofa"
    data, rpos, spos = _sofa_like(path, rng)
    s = read_sofa(path)
    assert s.GLOBAL_DataType == "TF" and not hasattr(s, "M")  # the bare dimension is left out
    assert s.ReceiverPosition_Type == "cartesian" and s.SourcePosition_Type == "spherical"
    d, src, rcv = convert_sofa(s)
    npt.assert_array_equal(d.freq, data + 0j)
    npt.assert_array_equal(d.frequencies, [125.0, 250.0, 500.0])
    npt.assert_array_equal(rcv.cartesian, rpos)
    az, el = np.deg2rad(spos[:, 0]), np.deg2rad(spos[:, 1])
    npt.assert_allclose(src.cartesian, np.stack([np.cos(el) * np.cos(az), np.cos(el) * np.sin(az), np.sin(el)], 1),
                        atol=1e-15)


def test_directional_wall_from_an_earliest_layout_file(tmp_path):
    from sparrowpy_gb300.geometry import shoebox_room_stub
    from sparrowpy_gb300.kang import PatchesDirectionalKang
    rng = np.random.default_rng(6)
    path = tmp_path / "brdf.sofa"
    data, _, _ = _sofa_like(path, rng)
    wall = shoebox_room_stub(1, 1, 1)[0]
    p = PatchesDirectionalKang.from_sofa(wall, 0.5, [], 0, path)
    npt.assert_allclose(p.directivity_data.freq, np.abs(data) * np.pi)
    npt.assert_array_equal(p.directivity_sources.weights, np.full(5, 0.2))
    assert p.n_dirs == 7


def test_malformed_file_raises(tmp_path):
    import pytest
    bad = tmp_path / "bad.sofa"
    bad.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes([9]) + bytes(200))
    with pytest.raises(NotImplementedError):
        hdf5.File(bad)
    bad.write_bytes(b"not hdf5")
    with pytest.raises(ValueError):
        hdf5.File(bad)


def test_version4_chunk_indexes(tmp_path):
    """Layout messages of version 4 (files of newer HDF5 releases): single-chunk (plain and filtered),
    implicit and fixed-array (plain and filtered) chunk indexes."""
    rng = np.random.default_rng(7)
    a = rng.normal(size=(5, 7))
    w = Writer()
    links = {"single": w.dataset(a, "v4-single"), "single_z": w.dataset(a, "v4-single", filters=True),
             "implicit": w.dataset(a, "v4-implicit", chunks=(2, 3)),
             "fixed": w.dataset(a, "v4-fixed", chunks=(2, 3)),
             "fixed_z": w.dataset(a, "v4-fixed", chunks=(2, 3), filters=True),
             "ints": w.dataset(np.arange(35, dtype=np.int32).reshape(5, 7), "v4-fixed", chunks=(3, 4))}
    path = tmp_path / "v4.h5"
    w.finish(path, links)
    ds = hdf5.File(path).datasets()
    for name in ("single", "single_z", "implicit", "fixed", "fixed_z"):
        npt.assert_array_equal(ds[name].read(), a, err_msg=name)
    npt.assert_array_equal(ds["ints"].read(), np.arange(35).reshape(5, 7))
