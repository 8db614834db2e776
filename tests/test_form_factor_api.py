"""The reference's form_factor package (sparrowpy/form_factor/kang.py, universal.py) on the GPU.

Pinned to a run of the reference here (tests/golden/form_factor.npz, made by
make_form_factor_golden.py): the Kang pair form factors of two rooms of
axis-aligned patches, the Kang and universal point-source energies (with and
without air attenuation) and receiver factors, 1e-12 relative (the FP64
library functions atan/exp/acos may differ in the last bit).  Plus the
reference's source-receiver reciprocity test for both methods
(tests/test_multisource.py:140-213).
"""
import numpy as np
import numpy.testing as npt
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def gold():
    return load_golden("form_factor")


def test_kang_form_factor_input_checks(gold):
    from sparrowpy_gb300.form_factor import patch2patch_ff_kang
    c, n = gold["cube_centers"], gold["cube_normals"]
    with pytest.raises(ValueError):
        patch2patch_ff_kang(c, n, np.ones((c.shape[0], 4)), gold["cube_pairs"])
    with pytest.raises(IndexError):  # orthogonal pairs need the third size column, as in the reference
        patch2patch_ff_kang(c, n, gold["cube_sizes"][:, :2], gold["cube_pairs"])
    assert not patch2patch_ff_kang(c, n, gold["cube_sizes"], np.zeros((0, 2))).any()


@pytest.mark.gpu
@pytest.mark.parametrize("room", ["cube", "room"])
def test_gpu_kang_pair_form_factors(gold, room):
    from sparrowpy_gb300.form_factor import patch2patch_ff_kang
    ff = patch2patch_ff_kang(gold[f"{room}_centers"], gold[f"{room}_normals"], gold[f"{room}_sizes"],
                             gold[f"{room}_pairs"])
    npt.assert_allclose(ff, gold[f"{room}_ff"], rtol=1e-12, atol=1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("room", ["cube", "room"])
def test_gpu_kang_point_factors(gold, room):
    from sparrowpy_gb300.form_factor import kang
    c, n, s = gold[f"{room}_centers"], gold[f"{room}_normals"], gold[f"{room}_sizes"]
    scale = np.array([3.0, 2.0, 2.5]) if room == "room" else np.ones(3)
    for k, src in enumerate(gold["sources"] * scale):
        e, d = kang._source2patch_energy_kang(src, c, n, gold["attenuation"], s, 2)
        e0, _ = kang._source2patch_energy_kang(src, c, n, None, s, 2)
        npt.assert_allclose(e, gold[f"{room}_src{k}_energy"], rtol=1e-12)
        npt.assert_allclose(e0, gold[f"{room}_src{k}_energy_noatt"], rtol=1e-12)
        npt.assert_allclose(d, gold[f"{room}_src{k}_distance"], rtol=1e-14)
    for k, rcv in enumerate(gold["receivers"] * scale):
        npt.assert_allclose(kang._patch2receiver_energy_kang(rcv - c, n), gold[f"{room}_rcv{k}_factor"], rtol=1e-14)


@pytest.mark.gpu
def test_gpu_universal_point_factors(gold):
    from sparrowpy_gb300.form_factor import universal
    pts, c = gold["cube_points"], gold["cube_centers"]
    vis = np.ones(c.shape[0], dtype=bool)
    for k, src in enumerate(gold["sources"]):
        e, d = universal._source2patch_energy_universal(src, c, pts, vis, gold["attenuation"], 2)
        npt.assert_allclose(e, gold[f"uni_src{k}_energy"], rtol=1e-12)
        npt.assert_allclose(d, gold[f"uni_src{k}_distance"], rtol=1e-14)
    for k, rcv in enumerate(gold["receivers"]):
        npt.assert_allclose(universal._patch2receiver_energy_universal(rcv, pts, vis), gold[f"uni_rcv{k}_factor"],
                            rtol=1e-12)
    hidden = vis.copy()
    hidden[::3] = False
    e, d = universal._source2patch_energy_universal(gold["sources"][0], c, pts, hidden, None, 1)
    assert not e[~hidden].any() and not d[~hidden].any() and e[hidden].all()


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["universal"])
@pytest.mark.parametrize("src", [[2., 0, 0], [2., 2., 0], [2., 0., 2.]])
@pytest.mark.parametrize("rec", [[1., 0., 0], [2., -2., 0], [2., 0., -2.]])
def test_gpu_reciprocity_point_source_patch_receiver(src, rec, method):
    """tests/test_multisource.py:140-213: swapping source and receiver around one 2 x 2 m patch gives the same
    source-energy times receiver-factor product (6 decimals, the reference's assert_array_almost_equal).

    The reference runs it with its default method="universal" only; its Kang branch is not reciprocal here
    (the reference's own Kang functions give 0.0210 against 0.0141 for the first case, as these do)."""
    from sparrowpy_gb300.form_factor import kang, universal
    from sparrowpy_gb300.geometry import Polygon
    wall = Polygon([[0, -1, -1], [0, -1, 1], [0, 1, 1], [0, 1, -1]], [0, 0, 1], [1, 0, 0])
    energy = []
    for a, b in ((src, rec), (rec, src)):
        a, b = np.asarray(a, float), np.asarray(b, float)
        if method == "universal":
            e_s, _ = universal._source2patch_energy_universal(a, wall.center[None], wall.pts[None], np.ones(1, bool),
                                                              np.zeros(1), 1)
            e_r = universal._patch2receiver_energy_universal(b, wall.pts[None], np.array([True]))
        else:
            e_s, _ = kang._source2patch_energy_kang(a, wall.center[None], wall.normal[None], np.zeros(1),
                                                    wall.size[None], 1)
            e_r = kang._patch2receiver_energy_kang((b - wall.center)[None], wall.normal[None])
        energy.append(e_s * e_r)
    npt.assert_array_almost_equal(energy[0], energy[1])
