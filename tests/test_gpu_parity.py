"""GPU parity: every step of the path, through the C ABI, against the golden vectors and the oracle.

Tolerances (per the path's specification):
  visibility, visible-pair list, outgoing-direction map: exact;
  form factors: rel <= 1e-10 (fp64), <= 1e-5 (fp32 Stokes; FP64 pairs <= 1e-10);
  receiver/patch histograms: rel L2 <= 1e-4 (fp32), <= 1e-10 (fp64).
"""
import numpy as np
import pytest

from conftest import acoustics, load_golden, radiosity_from_golden, rel_l2, scene_from_golden
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

SCENES = ["cube", "shoebox_126", "rot", "tri"]


def _solve(g, precision, algorithm="auto"):
    from sparrowpy_gb300.coords import Coordinates
    r = radiosity_from_golden(g, precision)
    c, dt, duration, k = acoustics(g)
    r.bake_geometry()
    r.init_source_energy(Coordinates(*g["source"]))
    r.calculate_energy_exchange(c, dt, duration, k, algorithm=algorithm)
    rc = g["receivers"]
    mono = r.collect_energy_receiver_mono(Coordinates(rc[:, 0], rc[:, 1], rc[:, 2])).time
    return r, mono


@pytest.fixture(scope="module", params=SCENES)
def golden(request):
    return load_golden(request.param)


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_bake_geometry(golden, precision):
    from sparrowpy_gb300.coords import Coordinates
    r = radiosity_from_golden(golden, precision)
    r.bake_geometry()
    np.testing.assert_array_equal(r._visibility_matrix, golden["V"])
    np.testing.assert_array_equal(r._visible_patches, golden["visible_patches"])
    np.testing.assert_array_equal(r._patch_2_brdf_outgoing_index, golden["p2o"].astype(np.int64))
    ff = r._form_factors[golden["visible_patches"][:, 0], golden["visible_patches"][:, 1]]
    method = r._bake["ff_method"].cpu().numpy()[: ff.size]
    rel = np.abs(ff - golden["ff_pairs"]) / np.abs(golden["ff_pairs"])
    assert rel[method != 0].max(initial=0) < 1e-10
    if precision == "fp32":
        assert rel[method == 0].max(initial=0) < 1e-5
    else:
        assert (method != 0).all()
    fft = r._form_factors_tilde
    tol = 1e-10 if precision == "fp64" else 1e-5
    if "ff_tilde" in golden:
        np.testing.assert_allclose(fft, golden["ff_tilde"], rtol=tol, atol=1e-300)
    else:
        sel = golden["ff_tilde_pairs"]
        np.testing.assert_allclose(fft[sel[:, 0], sel[:, 1]], golden["ff_tilde_sel"][0], rtol=tol)
        np.testing.assert_allclose(fft[sel[:, 1], sel[:, 0]], golden["ff_tilde_sel"][1], rtol=tol)


def test_source_energy(golden):
    from sparrowpy_gb300.coords import Coordinates
    r = radiosity_from_golden(golden, "fp64")
    r.bake_geometry()
    r.init_source_energy(Coordinates(*golden["source"]))
    np.testing.assert_array_equal(r._source_visibility, golden["svis"])
    np.testing.assert_allclose(r._distance_patches_to_source, golden["d0"], rtol=1e-15)
    np.testing.assert_allclose(r._energy_init_source, golden["e0dir"], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("precision,algorithm", [("fp64", "auto"), ("fp64", "dense"), ("fp32", "auto"),
                                                 ("fp32", "dense")])
def test_exchange_and_collect(golden, precision, algorithm):
    r, mono = _solve(golden, precision, algorithm)
    tol = 1e-10 if precision == "fp64" else 1e-4
    assert rel_l2(mono, golden["mono"]) < tol
    etot = r._energy_exchange_etc
    if "etot" in golden:
        assert rel_l2(etot, golden["etot"]) < tol
    else:
        assert rel_l2(etot[golden["etot_rows_index"]], golden["etot_rows"]) < tol
        assert rel_l2(etot.sum(axis=-1), golden["etot_time_sum"]) < tol


def test_patchwise_and_direct_sound(golden):
    from sparrowpy_gb300.coords import Coordinates
    r, mono = _solve(golden, "fp64")
    rc = golden["receivers"]
    rcv = Coordinates(rc[:, 0], rc[:, 1], rc[:, 2])
    pw = r.collect_energy_receiver_patchwise(rcv).time
    np.testing.assert_allclose(pw.sum(axis=1), golden["mono"], rtol=1e-9, atol=1e-300)
    # the private helper behind it (RadiosityFast.py:686-752): with propagation it is the patchwise
    # result; without, delaying each patch by ceil(d / c / dt) and attenuating it gives that result
    np.testing.assert_array_equal(r._collect_energy_patches(rc, propagation_fx=True), pw)
    raw = r._collect_energy_patches(rc)
    att = np.zeros(r.n_bins) if r._air_attenuation is None else np.asarray(r._air_attenuation, float)
    c, dt = r.speed_of_sound, r._etc_time_resolution
    expect = np.empty_like(raw)
    for i in range(rc.shape[0]):
        for k in range(r.n_patches):
            d = np.linalg.norm(r.patches_center[k] - rc[i])
            expect[i, k] = np.roll(raw[i, k] * np.exp(-att * d)[:, None], int(np.ceil(d / c / dt)), axis=-1)
    assert rel_l2(expect, pw) < 1e-12
    ds, delay = r.calculate_direct_sound(rcv)
    np.testing.assert_allclose(ds, golden["direct"], rtol=1e-14)
    np.testing.assert_array_equal(delay, golden["direct_delay"])
    with_ds = r.collect_energy_receiver_mono(rcv, direct_sound=True).time
    expect = golden["mono"].copy()
    expect[np.arange(rc.shape[0]), :, golden["direct_delay"]] += golden["direct"]
    assert rel_l2(with_ds, expect) < 1e-10


def test_oracle_agreement_seeded_per_patch_room():
    """A per-patch-material shoebox (one wall per patch, 0.5 m) against the oracle."""
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.coords import Coordinates
    from oracle.scene import scene_from_radiosity
    for precision in ("fp32", "fp64"):
        r = scenes.shoebox(0.5, n_dirs=8, n_bins=2, scattering=0.3, per_patch=True, seed=5, dims=(2.5, 2.0, 1.5),
                           air_attenuation=[0.001, 0.003], precision=precision)
        src, rcv = np.array([0.7, 0.6, 0.8]), np.array([[1.9, 1.3, 0.5]])
        c, dt, dur, k = 343.0, 1e-3, 0.12, 8
        r.bake_geometry()
        r.init_source_energy(Coordinates(*src))
        r.calculate_energy_exchange(c, dt, dur, k)
        mono = r.collect_energy_receiver_mono(Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])).time
        ref = orc.solve(scene_from_radiosity(r), src, rcv, c, dt, dur, k)
        np.testing.assert_array_equal(r._visibility_matrix, ref["bake"]["vis"])
        tol = 1e-10 if precision == "fp64" else 1e-4
        assert rel_l2(mono, ref["mono"]) < tol
        assert rel_l2(r._energy_exchange_etc, ref["etot"]) < tol


def test_brdf_structure_matches_host():
    """sp_brdf_structure (device) against brdf_rows_host: same medians, deviations and scales, bit for bit."""
    import torch
    from sparrowpy_gb300 import _native as nat
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.radiosity import _ptr, _stream, brdf_rows_host
    cases = [scenes.rotated_room(dense_box=False)[0], scenes.rotated_room(dense_box=True)[0],
             scenes.shoebox(0.5, n_dirs=8, n_bins=3, scattering=0.3, per_patch=True, seed=4, dims=(2.0, 1.5, 1.0))]
    for r in cases:
        bs = r._brdf_device()
        S, Din, Dout = bs["n_slots"], bs["n_in"], bs["n_out"]
        B = bs["brdf"].shape[-1]
        out = dict(diff=torch.empty((S, Din, B), dtype=torch.float64, device="cuda"),
                   spec=torch.empty((S, Din, B), dtype=torch.float64, device="cuda"),
                   target=torch.empty((S, Din), dtype=torch.int32, device="cuda"),
                   scale=torch.empty((S, B), dtype=torch.float64, device="cuda"))
        n_irr = torch.empty((1,), dtype=torch.int32, device="cuda")
        wsz = nat.size("sp_brdf_structure_workspace")
        ws = torch.empty((wsz,), dtype=torch.uint8, device="cuda")
        nat.call("sp_brdf_structure", S, Din, Dout, B, _ptr(bs["brdf"]), 1e-12, _ptr(out["diff"]), _ptr(out["spec"]),
                 _ptr(out["target"]), _ptr(out["scale"]), _ptr(n_irr), _ptr(ws), wsz, _stream())
        diff, spec, target, scale, irregular = brdf_rows_host(bs["brdf_host"])
        assert (int(n_irr.item()) > 0) == irregular
        np.testing.assert_array_equal(out["diff"].cpu().numpy(), diff)
        np.testing.assert_array_equal(out["scale"].cpu().numpy(), scale)
        if not irregular:
            np.testing.assert_array_equal(out["target"].cpu().numpy(), target)
            np.testing.assert_array_equal(out["spec"].cpu().numpy(), spec)


@pytest.mark.parametrize("max_order", [0, 1, 2])
@pytest.mark.parametrize("partial_sums", [True, False])
@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("fp64", 1e-12)])
def test_lowest_orders(precision, tol, partial_sums, max_order):
    """Orders 0 (E_total = E_0, the initial energies alone), 1 and 2 on the cube, against the reference-run
    golden scene's oracle solve at the same order, in both sum forms."""
    from sparrowpy_gb300.coords import Coordinates
    g = load_golden("cube")
    c, dt, duration, _ = acoustics(g)
    r = radiosity_from_golden(g, precision)
    r.partial_sums = partial_sums
    r.bake_geometry()
    r.init_source_energy(Coordinates(*g["source"]))
    r.calculate_energy_exchange(c, dt, duration, max_order)
    rc = g["receivers"]
    mono = r.collect_energy_receiver_mono(Coordinates(rc[:, 0], rc[:, 1], rc[:, 2])).time
    ref = orc.solve(scene_from_golden(g), g["source"], rc, c, dt, duration, max_order)
    assert rel_l2(r._energy_exchange_etc, ref["etot"]) < tol
    assert rel_l2(mono, ref["mono"]) < tol


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp64", 1e-10)])
def test_seeded_rooms_of_varied_shapes(precision, tol, seed):
    """Seeded shoeboxes of varied sizes, patch sizes, direction counts, bands, bin widths and orders, with
    histogram lengths that are not multiples of 4 on odd seeds (the mix for any length), against the oracle."""
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.coords import Coordinates
    rng = np.random.default_rng(100 + seed)
    dims = tuple(float(x) for x in np.round(rng.uniform(2.0, 4.0, 3) * 2) / 2)
    patch = float(rng.choice([0.5, 1.0]))
    n_dirs, n_bins = int(rng.choice([8, 16])), int(rng.choice([1, 3]))
    r = scenes.shoebox(patch, n_dirs=n_dirs, n_bins=n_bins, scattering=float(rng.uniform(0.2, 0.9)),
                       per_patch=bool(seed % 3 == 0), seed=seed, dims=dims, alpha_range=(0.05, 0.4),
                       air_attenuation=list(rng.uniform(0.0, 0.005, n_bins)), precision=precision)
    dt = float(rng.choice([1e-3, 7e-4]))
    nt = int(rng.integers(150, 320)) | (1 if seed % 2 else 0)
    nt += (4 - nt % 4) % 4 if seed % 2 == 0 else 0
    k = int(rng.integers(2, 8))
    src = np.array(dims) * rng.uniform(0.2, 0.8, 3)
    rcv = np.array(dims) * rng.uniform(0.2, 0.8, (2, 3))
    c = 343.0
    duration = nt * dt
    r.bake_geometry()
    r.init_source_energy(Coordinates(*src))
    r.calculate_energy_exchange(c, dt, duration, k)
    assert r._energy_exchange_etc.shape[-1] == int(duration / dt)
    mono = r.collect_energy_receiver_mono(Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])).time
    ref = orc.solve(scene_from_radiosity(r), src, rcv, c, dt, duration, k)
    assert rel_l2(mono, ref["mono"]) < tol, (dims, patch, n_dirs, n_bins, dt, nt, k)
    assert rel_l2(r._energy_exchange_etc, ref["etot"]) < tol
