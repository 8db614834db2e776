"""The benchmarked exchange shape against the FP64 oracle.

The street-canyon benchmark runs the structured exchange with 2000-bin
histograms (two 1024-bin scatter windows, the second one partial), pair
delays of up to about 300 bins (far beyond the 45-bin spread of a source
group, so windows reach into the zero lead of the padded rows), many receiver
tiles per class and 50 orders (E_total taken two orders at a time).  These
tests put exactly those code paths against the oracle
(RadiosityFast.py:1073-1145 restated in oracle/oracle.cpp):

* a per-patch-material shoebox solved end to end with histograms of 2200 and
  2500 bins, delays up to 43 and 215 bins, 50 and 49 orders (the pairing
  order of the benchmark, and an unpaired last order), with E_total as the
  last partial sum (S_k = E_0 + M(S_{k-1})) and order by order: receiver
  histograms, E_total, and the bins past 2048 (third window) within rel L2
  1e-4 (FP32) and 1e-10 (FP64);
* the 5939-patch street canyon itself, two orders: 16 sampled destination
  rows of E_1 and E_2 recomputed by the oracle from the GPU's own previous
  state and pair data (p2o, incoming BRDF row, F', delays), within rel L2
  1e-4 per row, and E_total = E_0 + E_1 + E_2 on those rows within 1e-6.
"""
import numpy as np
import pytest

from conftest import rel_l2
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _room(precision):
    from sparrowpy_gb300 import scenes
    # low absorption, so that the last window's bins (after 50 orders) stay far above FP32's range limit
    return scenes.shoebox(1.0, n_dirs=16, n_bins=2, scattering=0.3, per_patch=True, seed=7, alpha_range=(0.02, 0.1),
                          air_attenuation=[0.0012, 0.0031], precision=precision)


@pytest.mark.parametrize("partial_sums", [True, False])
@pytest.mark.parametrize("dt,duration,k", [(5e-4, 1.1, 50), (1e-4, 0.25, 49)])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_long_histograms_match_oracle(precision, dt, duration, k, partial_sums):
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300.coords import Coordinates
    r = _room(precision)
    r.partial_sums = partial_sums
    src, rcv = np.array([2.0, 2.0, 1.5]), np.array([[3.0, 4.0, 1.5], [4.1, 1.2, 2.3]])
    c = 343.0
    r.bake_geometry()
    r.init_source_energy(Coordinates(*src))
    r.calculate_energy_exchange(c, dt, duration, k)
    st = r.exchange_stats
    nt = int(duration / dt)
    assert st["algorithm"] == "structured" and nt >= 2048 and st["partial_sums"] == partial_sums
    assert st["tiles"] > 1 and st["segments"] > st["tiles"]
    delays = (r._bake["dist"].cpu().numpy()[: r._bake["n_dir"]] / c / dt).astype(np.int64)
    assert delays.max() >= (200 if dt < 2e-4 else 40)  # up to 4.7 times the 45-bin group spread
    mono = r.collect_energy_receiver_mono(Coordinates(rcv[:, 0], rcv[:, 1], rcv[:, 2])).time
    ref = orc.solve(scene_from_radiosity(r), src, rcv, c, dt, duration, k)
    tol = 1e-10 if precision == "fp64" else 1e-4
    assert rel_l2(mono, ref["mono"]) < tol
    etot = r._energy_exchange_etc
    assert rel_l2(etot, ref["etot"]) < tol
    # the last window's bins (past 2048) on their own, where they hold energy FP32 can represent (at 1.1 s
    # with 50 orders the tail is about 1e-90 of the peak: every order has arrived long before)
    tail = ref["etot"][..., 2048:]
    if precision == "fp64" or np.linalg.norm(tail) > 1e-6 * np.linalg.norm(ref["etot"]):
        assert rel_l2(etot[..., 2048:], tail) < tol
    if dt < 2e-4:
        # 49 orders of ~80 bins reach past 2048: values near 1e-8 against a peak near 0.1, checked above
        assert np.linalg.norm(tail) > 1e-5 * np.linalg.norm(ref["etot"])


def test_canyon_two_orders_match_oracle_rows():
    import torch
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.coords import Coordinates
    cfg = scenes.config("street_canyon_5939", precision="fp32")
    r = cfg["radiosity"]
    c, dt = cfg["c"], cfg["dt"]
    nt = int(cfg["duration"] / dt)
    r.bake_geometry()
    r.init_source_energy(Coordinates(*cfg["source"]))
    n, nd, nb = r._dev["e0dir"].shape
    states = torch.empty((3, n, nd, nb, nt), dtype=torch.float32, device=r.device)
    r._run_exchange(c, dt, nt, 2, states=states, states_every=1)
    assert r.exchange_stats["algorithm"] == "structured"
    etot = r._dev["etc"]
    bk = r._bake
    p = int(bk["n_dir"])
    dst_off = bk["dst_off"].cpu().numpy()
    src = bk["src"].cpu().numpy()[:p]
    p2o = bk["out_dir"].cpu().numpy()[:p]
    s_in = bk["in_dir"].cpu().numpy()[:p]
    dist = bk["dist"].cpu().numpy()[:p]
    fprime = bk["fprime"].cpu().numpy()[:p]
    unit_len = bk["unit_len"].cpu().numpy()[:p]
    bs = bk["brdf"]
    slot = np.asarray(r._brdf_index)[np.asarray(r._patch_to_wall_ids)[src]].astype(np.int32)
    att = np.asarray(r._air_attenuation, float)
    att_fac = np.exp(-att[None, :] * unit_len[:, None])
    delay = (dist / c / dt).astype(np.int64)
    assert delay.max() > 200
    rows = np.arange(0, n, n // 16)[:16].astype(np.int32)
    sel = np.concatenate([np.arange(dst_off[j], dst_off[j + 1]) for j in rows])
    # compact the pairs of the sampled rows; each reads source row src * nd + p2o
    sub_off = np.zeros(n + 1, dtype=np.int64)
    sub_off[rows + 1] = dst_off[rows + 1] - dst_off[rows]
    sub_off = np.cumsum(sub_off)
    need = src[sel].astype(np.int64) * nd + p2o[sel]
    uniq, inv = np.unique(need, return_inverse=True)
    idx = torch.as_tensor(uniq, device=r.device)
    for k in (1, 2):
        prev = states[k - 1].reshape(n * nd, nb, nt).index_select(0, idx).cpu().numpy()
        ref = orc.exchange_rows_out(nd, nb, nt, prev, inv, sub_off, delay[sel], fprime[sel], att_fac[sel], slot[sel],
                                    s_in[sel], bs["brdf_host"], rows)
        got = states[k][torch.as_tensor(rows, device=r.device)].double().cpu().numpy()
        for q in range(rows.size):
            assert rel_l2(got[q], ref[q]) < 1e-4, (k, int(rows[q]))
    tot = sum(states[k][torch.as_tensor(rows, device=r.device)].double() for k in range(3)).cpu().numpy()
    got_tot = etot[torch.as_tensor(rows, device=r.device)].double().cpu().numpy()
    assert rel_l2(got_tot, tot) < 1e-6
