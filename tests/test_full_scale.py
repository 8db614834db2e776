"""Parity at the benchmark's full size: the 5939-patch street canyon.

The oracle cannot solve the whole workload, but it can compute sampled
rows of it in seconds:
* visibility rows, every pair of the row against every blocker as
  geometry.py:750-797 does (bit-exact);
* the form factors of those rows' visible pairs (universal.py:12-52):
  - FP32 Stokes pairs within 1e-5 relative;
  - Nusselt pairs (shared vertex) within 1e-10 relative;
  - FP64 Stokes pairs within 1e-10 relative, or within the rounding bound
    of the sum itself when it cancels: the Stokes sum of 256 logarithm terms
    (integration.py:38-114) for a far pair is up to 1e7 times smaller than
    the sum of its terms' magnitudes.  Two FP64 summation orders (the
    reference's and the warp's) then differ by about sqrt(256) 2^-53 times
    that magnitude sum; the test allows 4 sqrt(256) 2^-53 sum |W ln r|.
and the whole solve at this size: the FP32 receiver histograms against the
FP64 solve's (the benchmark reports the same error).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_ROWS = 16
BOOLE = np.array([7.0, 32.0, 12.0, 32.0, 7.0])


def _boundary(el):
    """The 16 Boole sample points of each quadrilateral (integration.py:639-649, npoints 5): (n, 16, 3)."""
    pts = np.zeros((el.shape[0], 16, 3))
    for a in range(16):
        s, k = a >> 2, a & 3
        p, q = el[:, s], el[:, (s + 1) & 3]
        pts[:, a] = p + (k * (q - p)) / 4
    return pts


def _weights(el, pts):
    """Boole weight vectors of the sample points (integration.py:88-112): (n, 16, 3)."""
    w = np.zeros_like(pts)
    for a in range(16):
        s, k = a >> 2, a & 3
        for seg, pos in [(s, k)] + ([((s + 3) & 3, 4)] if k == 0 else []):
            x0, x1, x4 = pts[:, 4 * seg], pts[:, 4 * seg + 1], pts[:, (4 * seg + 4) & 15]
            w[:, a] += np.where(np.abs(x4 - x0) > 1e-3, 2 * (x1 - x0) / 45 * BOOLE[pos], 0.0)
    return w


def stokes_magnitude(pts_i, pts_j, area_i):
    """sum_ab |(u_a . v_b) ln r_ab| / (2 pi A_i) for each pair: the scale of the Stokes sum's rounding."""
    pi, pj = _boundary(pts_i), _boundary(pts_j)
    ui, vj = _weights(pts_i, pi), _weights(pts_j, pj)
    r = np.linalg.norm(pi[:, :, None, :] - pj[:, None, :, :], axis=-1)
    w = np.einsum("nad,nbd->nab", ui, vj)
    return np.sum(np.abs(w * np.log(r)), axis=(1, 2)) / (2 * np.pi * area_i)


def test_canyon_rows_match_oracle():
    from oracle import oracle as orc
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300 import scenes
    r = scenes.street_canyon(seed=3)
    n = r.n_patches
    r.bake_geometry()
    v = r._visibility_matrix
    sc = scene_from_radiosity(r)
    pts = sc["patches_points"]
    wall_of = np.asarray(sc["patch_to_wall_ids"])
    normals = sc["walls_normal"][wall_of]
    ctr = orc.centers(pts)
    stride = n // N_ROWS
    row_ids = np.arange(0, stride * N_ROWS, stride)
    _, rows = orc.visibility_rows_sample(ctr, normals, pts, 0, stride * N_ROWS, stride, full=True)
    sym = v | v.T
    for k, i in enumerate(row_ids):
        np.testing.assert_array_equal(rows[k].astype(bool), sym[i], err_msg=f"visibility row {i}")
    # form factors of the sampled rows' visible pairs (i < j)
    pairs = r._bake["pairs"].cpu().numpy()
    ff = r._bake["ff"].cpu().numpy()[: pairs.shape[0]]
    method = r._bake["ff_method"].cpu().numpy()[: pairs.shape[0]]
    sel = np.isin(pairs[:, 0], row_ids)
    assert sel.sum() > 1000
    ps, got, m = pairs[sel], ff[sel], method[sel]
    area = orc.areas(pts)
    ref = orc.form_factors(pts, normals, area, ps)
    err = np.abs(got - ref)
    rel = err / np.abs(ref)
    assert rel[m == 0].max(initial=0) < 1e-5, "FP32 Stokes"
    assert rel[m == 2].max(initial=0) < 1e-10, "Nusselt"
    s64 = m == 1
    bound = 1e-10 * np.abs(ref[s64]) + 4 * 16 * 2.0 ** -53 * stokes_magnitude(
        pts[ps[s64, 0]], pts[ps[s64, 1]], area[ps[s64, 0]])
    assert np.all(err[s64] <= bound), "FP64 Stokes"
    # most pairs stay on the FP32 path
    assert np.mean(m == 0) > 0.9


def test_canyon_fp32_solve_matches_fp64():
    """The whole 5939-patch solve (8 bands, 32 directions, 2000 bins, order 50): the FP32 receiver histograms
    within the 1e-4 relative L2 tolerance of the FP64 solve, itself parity-tested against the oracle at 1e-10."""
    import torch
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.coords import Coordinates

    def run(precision):
        c = scenes.config("street_canyon_5939", precision=precision)
        r = c["radiosity"]
        r.bake_geometry()
        r.init_source_energy(Coordinates(*c["source"]))
        r.calculate_energy_exchange(c["c"], c["dt"], c["duration"], c["max_order"])
        rc = c["receivers"]
        out = r.collect_energy_receiver_mono(Coordinates(rc[:, 0], rc[:, 1], rc[:, 2])).time
        del r, c
        torch.cuda.empty_cache()
        return out

    m32 = run("fp32")
    m64 = run("fp64")
    assert m32.shape == m64.shape == (8, 8, 2000)
    assert np.all(np.isfinite(m32)) and np.sum(m64) > 0
    assert np.linalg.norm(m32 - m64) / np.linalg.norm(m64) < 1e-4
