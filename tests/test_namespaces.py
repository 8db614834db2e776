"""The reference's public names (sparrowpy/__init__.py), and its form_factor entry points on the GPU
(form_factor/universal.py:12-96) against the reference's own integrals (tests/golden/polygons.npz)."""
import numpy as np
import pytest

import sparrowpy_gb300 as sp
from conftest import load_golden


def test_reference_public_names():
    for name in ("geometry", "sound_object", "DirectionalRadiosityFast", "RadiosityKang", "DirectionalRadiosityKang",
                 "PatchesKang", "PatchesDirectionalKang", "form_factor", "testing", "brdf", "utils"):
        assert hasattr(sp, name), name
    assert callable(sp.testing.shoebox_room_stub) and len(sp.testing.shoebox_room_stub(1, 2, 3)) == 6
    assert callable(sp.form_factor.patch2patch_ff_universal) and callable(sp.form_factor.patch2patch_ff_kang)
    assert callable(sp.form_factor.universal.universal_form_factor)
    assert callable(sp.brdf.create_from_scattering) and callable(sp.brdf.create_from_directional_scattering)
    assert callable(sp.utils.blender.read_geometry_file)
    assert callable(sp.geometry.Polygon) and callable(sp.sound_object.SoundSource)


@pytest.mark.gpu
@pytest.mark.parametrize("nv", [3, 5, 6])
def test_patch2patch_ff_universal(nv):
    g = load_golden("polygons")
    sel = np.flatnonzero((g["nvi"] == nv) & (g["nvj"] == nv))
    pts = np.concatenate([np.stack([g["pi"][k, :nv], g["pj"][k, :nv]]) for k in sel])
    normals = np.concatenate([np.stack([g["ni"][k], g["nj"][k]]) for k in sel])
    areas = np.repeat(g["area_i"][sel], 2)
    pairs = np.stack([2 * np.arange(sel.size), 2 * np.arange(sel.size) + 1], axis=1)
    ff = sp.form_factor.patch2patch_ff_universal(pts, normals, areas, pairs)
    assert ff.shape == (pts.shape[0],) * 2
    np.testing.assert_allclose(ff[pairs[:, 0], pairs[:, 1]], g["value"][sel], rtol=1e-10)
    mask = np.ones_like(ff, bool)
    mask[pairs[:, 0], pairs[:, 1]] = False
    assert not ff[mask].any()
    k = sel[0]
    one = sp.form_factor.universal.universal_form_factor(g["pi"][k, :nv], g["ni"][k], g["area_i"][k],
                                                         g["pj"][k, :nv], g["nj"][k])
    assert abs(one - g["value"][k]) <= 1e-10 * abs(g["value"][k])
