"""Host-side logic on CPU: patching, BRDF construction, BRDF structure analysis, API validation."""
import numpy as np
import pytest

from conftest import load_golden
import sparrowpy_gb300 as sp
from sparrowpy_gb300 import analyse_brdf, geometry, scenes
from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions, sph_gaussian
from sparrowpy_gb300.coords import Coordinates, FrequencyData
from oracle.scene import scene_from_radiosity


@pytest.mark.parametrize("name", ["cube", "shoebox_126"])
def test_patching_matches_reference(name):
    """geometry.py:290-410 `_process_patches` (golden patches from the reference run)."""
    g = load_golden(name)
    walls = g["walls_points"]
    size = {"cube": 0.5, "shoebox_126": 1.0}[name]
    pp, _, n, p2w = geometry.process_patches(walls, g["walls_normal"], size)
    np.testing.assert_array_equal(pp, g["patches_points"])
    np.testing.assert_array_equal(p2w, g["patch_to_wall_ids"])
    np.testing.assert_array_equal(geometry.calculate_center(pp), g["centers"])
    np.testing.assert_allclose(geometry.calculate_area(pp), g["areas"], rtol=1e-15)


@pytest.mark.parametrize("name", ["cube", "shoebox_126"])
def test_create_from_scattering_matches_reference(name):
    """brdf.py:8-130 run by the reference on the same directions."""
    g = load_golden(name)
    if "brdf_reference" not in g:
        pytest.skip("no BRDF pin in this fixture")
    p = g["brdf_params"]
    nb = (p.size - 1) // 2
    s, alpha, freqs = p[0], p[1:1 + nb], p[1 + nb:]
    dirs = Coordinates.from_cartesian(g["brdf_dirs"], weights=g["brdf_weights"])
    mine = create_from_scattering(dirs, dirs, FrequencyData(np.full(nb, s), freqs), FrequencyData(alpha, freqs))
    np.testing.assert_allclose(mine.freq, g["brdf_reference"], rtol=1e-12, atol=1e-15)


def test_scene_inputs_reproducible():
    """The host builders regenerate the stored golden inputs."""
    g = load_golden("shoebox_126")
    r = scenes.config("shoebox_126")["radiosity"]
    sc = scene_from_radiosity(r)
    np.testing.assert_allclose(sc["dirs_in"], g["dirs_in"], atol=1e-14)
    np.testing.assert_allclose(sc["dirs_out"], g["dirs_out"], atol=1e-14)
    np.testing.assert_allclose(sc["brdf"], g["brdf"], rtol=1e-13)


def test_wall_frame_half_space():
    """Rotated BRDF directions lie in the wall's half space (tests/test_DRadiosityFast.py:153-197)."""
    walls = sp.shoebox_room_stub(1, 1, 1)
    r = sp.DirectionalRadiosityFast.from_polygon(walls, 0.2)
    g = sph_gaussian(sh_order=1)
    d = Coordinates.from_cartesian(g.cartesian[g.z > 0], weights=g.weights[g.z > 0])
    data = create_from_scattering(d, d, FrequencyData(np.ones(4), [125, 250, 500, 1000]))
    r.set_wall_brdf([0, 1, 2], data, d, d)
    r.set_wall_brdf([3, 4, 5], data, d, d)
    assert len(r._brdf) == 2
    np.testing.assert_array_equal(r._brdf_index[:3], 0)
    np.testing.assert_array_equal(r._brdf_index[3:], 1)
    for b in r._brdf:
        assert b.shape == (4, 4, 4)
        np.testing.assert_allclose(b, 1.0)
    for i in range(6):
        assert (np.sum(r._brdf_incoming_directions[i].cartesian * r.walls_normal[i], axis=-1) > 0).all()
        assert (np.sum(r._brdf_outgoing_directions[i].cartesian * r.walls_normal[i], axis=-1) > 0).all()


def test_shapes_and_counts():
    """tests/test_DRadiosityFast.py:10-16 and :199-214."""
    r = sp.DirectionalRadiosityFast.from_polygon(sp.shoebox_room_stub(1, 1, 1), 0.5)
    assert r.patches_points.shape == (24, 4, 3)
    assert r.patches_area.shape == (24,)
    assert r.patches_center.shape == (24, 3)
    assert r.patches_size.shape == (24, 3)
    assert r.patches_normal.shape == (24, 3)
    assert geometry.total_number_of_patches(np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]]), 0.2) == 25


def test_air_attenuation_and_validation():
    r = sp.DirectionalRadiosityFast.from_polygon(sp.shoebox_room_stub(1, 1, 1), 0.2)
    r.set_air_attenuation(FrequencyData([0.1, 0.2], [500, 1000]))
    np.testing.assert_array_equal(r._air_attenuation, [0.1, 0.2])
    with pytest.raises(AssertionError, match="Number of frequency bins do not match"):
        r.set_air_attenuation(FrequencyData([0.1], [500]))
    with pytest.raises(ValueError, match="direct_sound must be of type boolean"):
        r.collect_energy_receiver_mono(Coordinates(0.5, 0.5, 0.5), direct_sound=1)
    with pytest.raises(ValueError, match="Receiver positions must be of type pf.Coordinates"):
        r.collect_energy_receiver_patchwise(np.zeros(3))
    with pytest.raises(ValueError, match="patch_to_wall_ids"):
        sp.DirectionalRadiosityFast(r.walls_points, r.walls_normal, r.walls_up_vector, r.patches_points,
                                    r.n_patches, np.zeros(r.n_patches + 1))
    d = hemisphere_directions(4)
    bad = Coordinates(0, 0, -1, weights=1)
    with pytest.raises(AssertionError, match="positive half space"):
        r.set_wall_brdf([0], FrequencyData(np.ones((1, 4, 2)), [500, 1000]), bad, d)


def test_analyse_brdf_reconstructs_tables():
    d = hemisphere_directions(16)
    freqs = np.array([125., 250., 500.])
    tabs = []
    for s, a in [(0.3, 0.1), (0.3, 0.4), (0.8, 0.2)]:
        tabs.append(np.pi * create_from_scattering(d, d, FrequencyData(np.full(3, s), freqs),
                                                   FrequencyData(np.full(3, a), freqs)).freq)
    brdf = np.array(tabs)
    st = analyse_brdf(brdf)
    assert st is not None and st["n_groups"] == 2
    S, Din, Dout, B = brdf.shape
    for slot in range(S):
        g = st["slot_group"][slot]
        for s in range(Din):
            c = g * Din + s
            row = st["class_diff"][c][None, :] * np.ones((Dout, 1))
            if st["class_target"][c] >= 0:
                row[st["class_target"][c]] += st["class_spec"][c]
            np.testing.assert_allclose(row * st["slot_scale"][slot], brdf[slot, s], rtol=1e-12)
    rng = np.random.default_rng(0)
    assert analyse_brdf(rng.uniform(size=(2, 8, 8, 2))) is None


def test_to_dict_round_trip():
    r = sp.DirectionalRadiosityFast.from_polygon(sp.shoebox_room_stub(2, 2, 2), 1.0)
    d = hemisphere_directions(4)
    r.set_wall_brdf(np.arange(6), create_from_scattering(d, d, FrequencyData([0.5], [500])), d, d)
    r.set_air_attenuation(FrequencyData([0.0], [500]))
    r2 = sp.DirectionalRadiosityFast.from_dict(r.to_dict())
    assert r2.n_patches == r.n_patches
    np.testing.assert_array_equal(r2.patches_points, r.patches_points)
    np.testing.assert_array_equal(r2._air_attenuation, r._air_attenuation)


def test_material_tables_reproduce_create_from_scattering():
    """The adjoint's material parametrisation is create_from_scattering x pi (brdf.py:8-130, RadiosityFast.py:815)."""
    import torch
    from sparrowpy_gb300.adjoint import material_tables, mirror_table
    from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions
    from sparrowpy_gb300.coords import FrequencyData
    dirs = hemisphere_directions(16)
    mirror, gain = mirror_table(dirs)
    assert (mirror >= 0).all()
    rng = np.random.default_rng(1)
    alpha = rng.uniform(0.0, 0.6, (3, 4))
    scat = rng.uniform(0.0, 1.0, (3, 4))
    tabs = material_tables(torch.tensor(alpha), torch.tensor(scat), mirror, gain, 16).numpy()
    freqs = np.array([125.0, 250.0, 500.0, 1000.0])
    for k in range(3):
        ref = np.asarray(create_from_scattering(dirs, dirs, FrequencyData(scat[k], freqs),
                                                FrequencyData(alpha[k], freqs)).freq) * np.pi
        np.testing.assert_allclose(tabs[k], ref, rtol=1e-13, atol=1e-15)


def test_state_file_round_trip(tmp_path):
    """write / from_read (RadiosityFast.py:828-839) keep every host input, direction sets included."""
    r = sp.DirectionalRadiosityFast.from_polygon(sp.shoebox_room_stub(2, 3, 2), 1.0)
    d = hemisphere_directions(4)
    f = np.array([500.0, 1000.0])
    r.set_wall_brdf(np.arange(3), create_from_scattering(d, d, FrequencyData([0.5, 0.4], f)), d, d)
    r.set_wall_brdf(np.arange(3, 6), create_from_scattering(d, d, FrequencyData([0.2, 0.1], f)), d, d)
    r.set_air_attenuation(FrequencyData([0.001, 0.002], f))
    r.write(tmp_path / "state.far")
    r2 = sp.DirectionalRadiosityFast.from_read(tmp_path / "state.far")
    assert r2 == r
    for a, b in zip(r._brdf_outgoing_directions, r2._brdf_outgoing_directions):
        np.testing.assert_array_equal(np.asarray(a.cartesian), np.asarray(b.cartesian))
        np.testing.assert_array_equal(a.weights, b.weights)
    assert len(r2._brdf) == 2 and r2._brdf_index.tolist() == r._brdf_index.tolist()


def test_state_file_reads_ndarray_and_builtin_members(tmp_path):
    """A pyfar-style file holding only ndarray and builtin members (the reference's own layout) reads back."""
    import io
    import json
    import zipfile
    from sparrowpy_gb300 import far
    arr = np.arange(12.0).reshape(3, 4)
    buf = io.BytesIO()
    np.save(buf, arr)
    path = tmp_path / "plain.far"
    with zipfile.ZipFile(path, "w") as z:
        z.writestr("E_matrix/$ndarray", buf.getvalue())
        z.writestr("builtin_wrapper/$BuiltinsWrapper", json.dumps({"pyfar.__version__": "0.6.5", "c": 343.0,
                                                                   "note": "None"}))
    vals = far.read(path)
    np.testing.assert_array_equal(vals["E_matrix"], arr)
    assert vals["c"] == 343.0 and vals["note"] == "None"
    with zipfile.ZipFile(path, "a") as z:
        z.writestr("src/$Coordinates", b"{}")
    with pytest.raises(NotImplementedError):
        far.read(path)


def test_pair_dir_tables_merge_identical_walls():
    """The pair set-up's merged direction tables: every wall maps to a table equal to its own."""
    import torch
    from sparrowpy_gb300.radiosity import _pair_dir_tables
    rng = np.random.default_rng(0)
    base_in = rng.standard_normal((3, 5, 3))
    base_out = rng.standard_normal((3, 7, 3))
    which = np.array([2, 0, 0, 1, 2, 2, 1, 0])  # 8 walls, 3 distinct orientations
    bs = dict(n_in=5, n_out=7, dirs_in=torch.tensor(base_in[which]), dirs_out=torch.tensor(base_out[which]))
    tab, din, dout = _pair_dir_tables(bs)
    assert din.shape == (3, 5, 3) and dout.shape == (3, 7, 3)
    tab = tab.numpy()
    np.testing.assert_array_equal(din.numpy()[tab], base_in[which])
    np.testing.assert_array_equal(dout.numpy()[tab], base_out[which])
    assert _pair_dir_tables(bs)[0] is bs["pair_tables"][0]  # cached with the state


def test_kang_form_factor_columns():
    """PatchesKang._column: offsets of the other walls' patches in other_wall_ids order (RadiosityKang.py:410-441)."""
    walls = geometry.shoebox_room_stub(2, 1, 1)
    radi = sp.RadiosityKang(walls, 0.5, 1, 0.1)
    p0 = radi.patch_list[0]
    sizes = [len(p.patches) for p in radi.patch_list]
    off = 0
    for w in p0.other_wall_ids:
        assert p0._column(radi.patch_list, w) == off
        off += sizes[w]
    with pytest.raises(KeyError):
        p0._column(radi.patch_list, 0)
