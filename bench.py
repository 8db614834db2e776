#!/usr/bin/env python
"""Benchmark: milliseconds per solve (bake + exchange) of the street-canyon workload.

Workload (default ``--config street_canyon_5939``): two 100 x 20 m facades 15 m apart and a
100 x 15 m ground, 1 m patches, 40 seeded box occluders (5939 patches, one
wall per patch), 8 octave bands, 32 directions, per-patch/per-band
absorption U[0.01, 0.3], scattering 0.3, 1 source and 8 receivers, 1 ms x
2 s histograms, reflection order 50.  Synthetic, seeded scene (no dataset).

A step is one solve: bake_geometry + init_source_energy +
calculate_energy_exchange (all orders) through sparrowpy_gb300's
DirectionalRadiosityFast.  ``value`` times it with every input already in
device memory (CUDA events on the solve's stream); ``e2e`` times the same
solve from host arrays through the public API, including the host->device
upload of the scene and the device->host read of the receiver histograms.
Every histogram array (12 GB for this workload) exceeds the 129 MB L2, so
no flush is needed between steps.

``--impl reference`` times the reference's loops on the host cores: the
FP64 C++/OpenMP restatement in oracle/ (the reference is Python + numba,
which is not installed here), on bounded samples of the same workload,
extrapolated to one solve.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
# the FP32 and FP64 solves each hold tens of GB of histograms and workspace;
# growable segments let the second reuse what the first released
if "PYTORCH_CUDA_ALLOC_CONF" not in os.environ:
    os.environ.setdefault("PYTORCH_ALLOC_CONF", "expandable_segments:True")

import numpy as np  # noqa: E402

METRIC = "ms/solve (bake+exchange) ~5.5k patches FP32 vs FP64 GPU; fwd+bwd ms; HBM GB/s"
PEAKS_FILE = os.path.join(HERE, "MEASURED_PEAKS.json")
# DRAM bytes moved per algorithmic byte by one exchange order (scatter, mix
# and source add of the partial sums, which read and write no E_total), from
# a single-pass ncu capture (dram__bytes_read.sum + dram__bytes_write.sum)
# of the 1759-patch canyon
TRAFFIC_PER_ALGO_BYTE = 0.81


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--config", default="street_canyon_5939")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--max-order", type=int, default=None, help="override the workload's reflection order")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU comparison solve")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-fwd-bwd", action="store_true", help="skip the gradient (forward + backward) leg")
    ap.add_argument("--no-configs", action="store_true", help="skip the shoebox_126 / shoebox_2016 legs")
    ap.add_argument("--no-kahan", action="store_true", help="skip the plain-sum solves that time the Kahan cost")
    ap.add_argument("--batch-rooms", type=int, default=256,
                    help="seeded shoebox rooms for the batch leg (256 by default; 0: skip)")
    ap.add_argument("--leg", default=None, choices=["general", "batch"],
                    help="print only one leg as one JSON line (profiling runs)")
    ap.add_argument("--general-patch", type=float, default=0.25,
                    help="patch size of the general-BRDF leg's room (1.0: 126 patches, a small profiling case)")
    ap.add_argument("--fwd-bwd-only", action="store_true",
                    help="print only the gradient leg (shoebox, 2016 patches) as one JSON line")
    return ap.parse_args()


# ------------------------------------------------------------------- helpers
def dist_env():
    from sparrowpy_gb300.replicas import env_ranks
    return env_ranks()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu = gpu_id  # UUID of the device, or None for every visible GPU
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi"] + ([f"--id={self.gpu}"] if self.gpu else []) +
                [f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                except ValueError:
                    continue
                for k, name in enumerate(names):
                    if f[5 + k].lower().startswith("active"):
                        reasons.add(name)
            os.unlink(self.path)
        except Exception:
            pass
        if sm:
            busy = [s for s in sm if s > 0.5 * max(sm)] or sm
            out = {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def nt_late(cfg):
    """First Kahan-compensated bin of E_total: half the histogram, on a multiple of 4."""
    return (int(round(cfg["duration"] / cfg["dt"])) // 2) & ~3


def algorithmic_bytes_per_order(n, d, b, t, pairs, n_slots, n_in, elem=4):
    """Algorithmic bytes of one exchange order in the reference's order-by-order form.

    4 x N D B T histogram elements (read E_{k-1}, write E_k, read and write
    E_total) + 16 bytes per directed pair (F', delay, directions) + one read
    of the BRDF tables (S Din D B, FP32).  The partial sums (the default)
    need only the first two of the four histogram terms; the figure keeps the
    reference form's count, so `roofline.traffic` falls below it.
    """
    return 4.0 * elem * n * d * b * t + 16.0 * pairs + 4.0 * n_slots * n_in * d * b


def peak_hbm():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# -------------------------------------------------------------- CPU baseline
def cpu_baseline(cfg, rows_per_thread=1, exchange_rows=8):
    """FP64 CPU restatement (oracle/) on bounded samples, extrapolated to one solve.

    GPU-free.  Each part runs on the threads the reference's numba code uses
    for it: visibility and form factors on every host thread (numba
    parallel=True, geometry.py:919, universal.py:164), the exchange on one
    (RadiosityFast.py:1396 compiles _energy_exchange with numba.njit(), not
    parallel).  Samples, all on the same scene and its own pair lists:
      visibility - full rows of the visibility matrix at evenly spaced
                   patches (every pair against every blocker, as
                   geometry.py:750-797), scaled by N(N-1)/2 / pairs evaluated;
      form factors - the visible pairs (i < j) of those rows (universal.py),
                   scaled by the visible-pair count those rows imply;
      exchange   - one order of RadiosityFast.py:1121-1143 for
                   `exchange_rows` of the sampled patches as destinations,
                   their visible partners as sources (true delays; source
                   rows read from a 64-row buffer, the cost does not depend on
                   the values), times N / rows and the number of orders.
    Returns (ms_per_solve, threads, description).
    """
    from oracle import oracle as orc
    from oracle.scene import scene_from_radiosity
    r = cfg["radiosity"]
    sc = scene_from_radiosity(r)
    n = r.n_patches
    threads = orc.num_threads()
    rng = np.random.default_rng(0)
    pts = sc["patches_points"]
    wall_of = np.asarray(sc["patch_to_wall_ids"])
    normals = sc["walls_normal"][wall_of]
    ctr = orc.centers(pts)
    area = orc.areas(pts)
    # visibility rows: a whole number of rows per thread, evenly spaced
    n_rows = max(2, min(n, threads * rows_per_thread))
    stride = max(1, n // n_rows)
    t0 = time.perf_counter()
    n_visible, rows = orc.visibility_rows_sample(ctr, normals, pts, 0, stride * n_rows, stride, full=True)
    t_vis = time.perf_counter() - t0
    row_ids = np.arange(0, stride * n_rows, stride)
    pairs_evaluated = rows.shape[0] * (n - 1)
    t_vis *= (n * (n - 1) / 2) / pairs_evaluated
    total_visible = n_visible / rows.shape[0] * n / 2  # unordered visible pairs of the scene
    # form factors of the sampled visible pairs (i < j)
    ii, jj = np.nonzero(rows)
    ii = row_ids[ii]
    keep = ii < jj
    pairs = np.stack([ii[keep], jj[keep]], axis=1).astype(np.int32)
    k = min(pairs.shape[0], 2500 * n_rows)
    pairs = pairs[rng.choice(pairs.shape[0], size=k, replace=False)] if k < pairs.shape[0] else pairs
    t0 = time.perf_counter()
    orc.form_factors(pts, normals, area, pairs)
    t_ff = (time.perf_counter() - t0) * total_visible / max(pairs.shape[0], 1)
    # one exchange order for some of the sampled rows as destinations
    keep_rows = np.linspace(0, rows.shape[0] - 1, min(exchange_rows, rows.shape[0])).astype(int)
    rows, row_ids = rows[keep_rows], row_ids[keep_rows]
    nd = sc["dirs_out"].shape[1]
    nb = sc["brdf"].shape[-1]
    n_in = sc["brdf"].shape[1]
    nt = int(cfg["duration"] / cfg["dt"])
    counts = rows.sum(axis=1).astype(np.int64)
    dst_off = np.zeros(n + 1, dtype=np.int64)
    dst_off[row_ids + 1] = counts
    dst_off = np.cumsum(dst_off)
    src = np.nonzero(rows)[1].astype(np.int32)
    dst = np.repeat(row_ids, counts)
    dist = np.linalg.norm(ctr[src] - ctr[dst], axis=1)
    delay = (dist / cfg["c"] / cfg["dt"]).astype(np.int32)
    m = src.size
    p2o = rng.integers(0, nd, m).astype(np.int32)
    s_in = rng.integers(0, n_in, m).astype(np.int32)
    fprime = rng.uniform(0, 1e-2, m)
    att = np.ones((m, nb))
    slot = np.asarray(sc["brdf_index"])[wall_of[src]].astype(np.int32)
    prev = rng.uniform(0, 1e-3, size=(64, nd * nb * nt))
    orc.set_threads(1)  # the reference's exchange is serial numba
    try:
        t0 = time.perf_counter()
        orc.exchange_rows_sample(nd, nb, nt, prev, dst_off, src, p2o, delay, fprime, att, slot, s_in, sc["brdf"],
                                 row_ids.astype(np.int32))
        t_order = (time.perf_counter() - t0) * n / rows.shape[0]
    finally:
        orc.set_threads(threads)
    total = t_vis + t_ff + cfg["max_order"] * t_order
    desc = (f"EXTRAPOLATED from samples (no complete solve at this size): oracle C++/OpenMP FP64, visibility and "
            f"form factors on {threads} threads (numba parallel=True in the reference), the exchange on 1 thread "
            f"(serial numba.njit in the reference, RadiosityFast.py:1396): visibility of {n_rows} full patch rows "
            f"({pairs_evaluated} pairs x {n} blockers), form factors of {pairs.shape[0]} of their visible pairs, "
            f"one exchange order for {rows.shape[0]} destination patches ({m} incoming pairs); "
            f"extrapolated by pair/row counts to one solve: visibility {t_vis:.1f} s, form factors {t_ff:.1f} s, "
            f"{cfg['max_order']} orders x {t_order:.1f} s")
    return total * 1e3, threads, desc


def cpu_full_solve_shoebox_126():
    """One complete oracle solve of the 126-patch shoebox, timed, no extrapolation.

    Bake (visibility and form factors on every host thread, as the
    reference's parallel numba loops), source energy, the 20 exchange orders
    on one thread (serial in the reference) and the receiver histogram.
    Returns (ms, threads, description, mono).
    """
    from oracle import oracle as orc
    from oracle.scene import scene_from_radiosity
    from sparrowpy_gb300 import scenes
    cfg = scenes.config("shoebox_126", precision="fp64")
    sc = scene_from_radiosity(cfg["radiosity"])
    threads = orc.num_threads()
    src, rcv = cfg["source"], cfg["receivers"]
    nt = int(cfg["duration"] / cfg["dt"])
    t0 = time.perf_counter()
    bk = orc.bake(sc)
    e0dir, d0, _ = orc.init_source(sc, bk, src)
    t1 = time.perf_counter()
    orc.set_threads(1)
    try:
        etot = orc.exchange(sc, bk, e0dir, d0, cfg["c"], cfg["dt"], nt, cfg["max_order"])
    finally:
        orc.set_threads(threads)
    t2 = time.perf_counter()
    mono = orc.collect(sc, bk, etot, rcv, cfg["c"], cfg["dt"])
    t3 = time.perf_counter()
    desc = (f"complete oracle FP64 solve of the 126-patch shoebox ({bk['src'].size} directed pairs, 16 directions, "
            f"1 band, T={nt}, order {cfg['max_order']}): bake + source {1e3 * (t1 - t0):.0f} ms on {threads} threads, "
            f"exchange {1e3 * (t2 - t1):.0f} ms on 1 thread, collection {1e3 * (t3 - t2):.0f} ms")
    return 1e3 * (t2 - t0), threads, desc, mono


# ----------------------------------------------------------------- GPU arm
def solve(r, cfg, coords):
    """One step: bake, source energy and every exchange order (the public API calls)."""
    r.bake_geometry()
    r.init_source_energy(coords(cfg["source"]))
    r.calculate_energy_exchange(cfg["c"], cfg["dt"], cfg["duration"], cfg["max_order"], recalculate=True)


def smem_roofline(stats, nb, nt, scatter_ms_total, sm_mhz):
    """The scatter's binding roofline: shared-memory wavefronts (128 B, one per SM cycle at most).

    Per (source group, band, 1024-bin window) the scatter reads 32 wavefronts
    per member (one 32-float window read per FMA slice), about 16.75 for the
    per-warp member words and coefficients, and writes 33.5 wavefronts of
    staged window (4288 bytes) by bulk copy.  The LSU part of this count
    matched the ncu counter of a captured launch within 4 %.
    """
    import torch
    if not scatter_ms_total or scatter_ms_total <= 0 or not sm_mhz:
        return None
    orders = max(stats["orders"], 1)
    windows = (nt + 1023) // 1024
    per_order = nb * windows * (32.0 * stats["pairs"] + (16.75 + 33.5) * stats["source_groups"])
    sec = scatter_ms_total / orders * 1e-3
    n_sm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    peak = n_sm * sm_mhz * 1e6
    return {"bound": "shared-memory", "kernel": "k_scatter_f32", "unit": "wavefronts/s",
            "achieved": per_order / sec, "peak": peak, "frac": per_order / sec / peak,
            "ms_per_launch": scatter_ms_total / orders, "wavefronts_per_launch": per_order,
            "model": "per (group, band, 1024-bin window): 32 per member + 16.75 words + 33.5 copy; "
                     "peak = SMs x median SM clock under load"}


def workload_config(name, cfg, world):
    r = cfg["radiosity"]
    nt = int(round(cfg["duration"] / cfg["dt"]))
    nb = len(r._frequencies)
    nd = r._brdf_outgoing_directions[0].cartesian.reshape(-1, 3).shape[0]
    desc = {"street_canyon_5939": "street canyon: 100 x 20 m facades 15 m apart + 100 x 15 m ground, 1 m patches, "
                                  "40 box occluders",
            "street_canyon_1759": "street canyon: 30 x 20 m facades 15 m apart + ground, 1 m patches, "
                                  "10 box occluders"}
    return {"workload": f"{desc.get(name, name)}; {r.n_patches} patches, {nb} bands, {nd} directions, "
                        f"{nt} x {cfg['dt'] * 1e3:g} ms bins, reflection order {cfg['max_order']}, 1 source",
            "name": name, "patches": r.n_patches, "bands": nb, "directions": nd, "bins": nt,
            "max_order": cfg["max_order"], "receivers": int(np.atleast_2d(cfg["receivers"]).shape[0]),
            "l2_policy": "inputs larger than L2 (each histogram array >= 1 GB), no flush",
            "value_state": "each timed solve re-runs bake, source and exchange on one object; it reuses that "
                           "object's uploaded BRDF tables, their grouping and the receiver tile order (e2e builds "
                           "a fresh object per step and includes them)",
            "parallelism": f"replicas x{world}"}


def as_coords(x):
    from sparrowpy_gb300.coords import Coordinates
    x = np.asarray(x, float)
    return Coordinates(*x.T) if x.ndim > 1 else Coordinates(*x)


def gpu_uuid(local):
    import torch
    try:
        u = str(torch.cuda.get_device_properties(local).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        return None


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from sparrowpy_gb300 import _native, scenes

    from sparrowpy_gb300.replicas import max_over_ranks
    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    cfg = scenes.config(args.config, precision=args.precision)
    if args.max_order is not None:
        cfg["max_order"] = args.max_order
    r = cfg["radiosity"]
    host_template = r.clone()
    st = torch.cuda.current_stream()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        solve(r, cfg, as_coords)
    barrier()
    clocks = ClockSampler(gpu_uuid(local))
    clocks.start()
    time.sleep(0.3)
    launches0 = _native.lib().sp_kernel_launches()
    times, order_ms, scatter_ms = [], [], []
    barrier()
    for _ in range(args.steps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(st)
        solve(r, cfg, as_coords)
        ev1.record(st)
        ev1.synchronize()
        times.append(ev0.elapsed_time(ev1))
        order_ms.append(r.exchange_stats["order_ms"])
        scatter_ms.append(r.exchange_stats["scatter_ms"])
    barrier()
    launches = _native.lib().sp_kernel_launches() - launches0
    clk = clocks.stop()
    ms_step = max_over_ranks(float(np.mean(times)))

    # end to end through the public API from host arrays: upload of the
    # scene and materials, bake, source, exchange, receiver histograms back
    # (one untimed step first: a fresh object's first allocations come from
    # cudaMalloc; later objects reuse the allocator's cache, as a user's
    # repeated solves do; every timed step still uploads all inputs)
    e2e_times, h2d, d2h = [], 0, 0
    for k in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        r2 = host_template.clone()
        barrier()
        t0 = time.perf_counter()
        solve(r2, cfg, as_coords)
        mono = r2.collect_energy_receiver_mono(as_coords(cfg["receivers"])).time
        torch.cuda.synchronize()
        if k > 0:
            e2e_times.append((time.perf_counter() - t0) * 1e3)
        h2d = int(r2.host_bytes_uploaded)
        d2h = int(mono.nbytes)
        del r2, mono
    e2e_ms = max_over_ranks(float(np.mean(e2e_times)) if e2e_times else None)

    # E_total as the last partial sum (the default, timed above) against the reference's order-by-order
    # sums, with the late bins Kahan-compensated and with plain FP32 sums: time and receivers of each
    monos = {"partial_sums": r.collect_energy_receiver_mono(as_coords(cfg["receivers"])).time}
    forms = {}
    for name, comp in ([] if args.no_kahan else [("order_sums_compensated", True), ("order_sums_plain", False)]):
        r.partial_sums, r.compensated_total = False, comp
        t = []
        for k in range(2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            solve(r, cfg, as_coords)
            e1.record(st)
            e1.synchronize()
            t.append((e0.elapsed_time(e1), r.exchange_stats["order_ms"]))
        forms[name] = {"ms_per_solve": float(np.mean([p[0] for p in t])),
                       "exchange_ms": float(np.mean([p[1] for p in t]))}
        monos[name] = r.collect_energy_receiver_mono(as_coords(cfg["receivers"])).time
    r.partial_sums, r.compensated_total = True, True
    sum_forms = None if not forms else {
        "default": "partial sums: S_k = E_0 + M(S_{k-1}), E_total = S_K",
        "partial_sums": {"ms_per_solve": ms_step, "exchange_ms": float(np.mean(order_ms))},
        **forms, "late_bins_from": int(nt_late(cfg)), "compensation_storage": "bfloat16 per late bin"}

    # roofline of one exchange order (scatter + mix launches of that order)
    stats = r.exchange_stats
    n, nd, nb, nt = r._dev["etc"].shape
    plan = r._bake["plan"]
    n_pairs = int(r._bake["n_dir"])
    bytes_order = algorithmic_bytes_per_order(n, nd, nb, nt, n_pairs, plan["n_slots"], plan["n_in"],
                                              elem=4 if args.precision == "fp32" else 8)
    ms_order = float(np.mean(order_ms)) / max(stats["orders"], 1)
    achieved = bytes_order / (ms_order * 1e-3) / 1e9
    peak, peak_kind = peak_hbm()
    smem = smem_roofline(stats, nb, nt, float(np.mean(scatter_ms)), clk.get("sm_mhz"))

    fp64 = None
    if not args.no_fp64 and args.precision == "fp32" and rank == 0:
        r._dev.pop("ws", None)  # the FP64 solve needs the room of the FP32 workspace
        torch.cuda.empty_cache()
        c64 = scenes.config(args.config, precision="fp64")
        c64["max_order"] = cfg["max_order"]
        r64 = c64["radiosity"]
        t64 = []  # one timed FP64 solve (about a minute; its first-use allocations are small against that)
        for _ in range(1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            solve(r64, c64, as_coords)
            e1.record(st)
            e1.synchronize()
            t64.append(e0.elapsed_time(e1))
        m64 = r64.collect_energy_receiver_mono(as_coords(cfg["receivers"])).time
        rel = lambda m: float(np.linalg.norm(m - m64) / np.linalg.norm(m64))
        fp64 = {"ms_per_solve": float(np.mean(t64)), "fp64_over_fp32": float(np.mean(t64)) / ms_step,
                "exchange_ms_per_order": r64.exchange_stats["order_ms"] / max(stats["orders"], 1),
                "receiver_rel_l2_fp32_vs_fp64": rel(monos["partial_sums"]),
                "receiver_rel_l2_fp32_vs_fp64_by_sum_form": {k: rel(m) for k, m in monos.items()}}
        del r64, c64
        torch.cuda.empty_cache()

    fwd_bwd = None
    if not args.no_fwd_bwd and rank == 0:
        r._dev.clear()  # the street canyon's device state; its host inputs stay for the CPU leg
        r._bake = None
        torch.cuda.empty_cache()
        try:
            fwd_bwd = fwd_bwd_config4()
        except Exception as exc:  # the gradient leg must not hide the solve result
            fwd_bwd = {"error": f"{type(exc).__name__}: {exc}"}

    configs = None
    if not args.no_configs and rank == 0:
        r._dev.clear()
        r._bake = None
        torch.cuda.empty_cache()
        try:
            shoebox_126_cpu = None if args.no_cpu else cpu_full_solve_shoebox_126()
            configs = config_legs(shoebox_126_cpu)
        except Exception as exc:  # the config legs must not hide the solve result
            configs = {"error": f"{type(exc).__name__}: {exc}"}

    general = None
    if not args.no_configs and rank == 0:
        try:
            general = general_brdf_leg()
        except Exception as exc:  # must not hide the solve result
            general = {"error": f"{type(exc).__name__}: {exc}"}

    batch = None
    if args.batch_rooms > 0:
        barrier()
        try:
            batch = batch_rooms(args.batch_rooms, rank=rank, world=world)
        except Exception as exc:  # the batch leg must not hide the solve result
            batch = {"error": f"{type(exc).__name__}: {exc}"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        try:
            ms_cpu, cores, desc = cpu_baseline(cfg, rows_per_thread=2)
            cpu = {"value": ms_cpu, "unit": "ms/solve", "cores": cores, "kind": "port", "sample": desc}
            if configs and "shoebox_126" in configs and "cpu_measured" in configs["shoebox_126"]:
                cpu["measured_shoebox_126"] = configs["shoebox_126"]["cpu_measured"]
        except Exception as exc:  # the CPU leg must not hide the GPU result
            cpu = {"value": None, "unit": "ms/solve", "cores": None, "kind": "port", "sample": f"failed: {exc}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": ms_step / world, "unit": "ms/solve", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else "f64",
            "data": "synthetic: seeded street-canyon geometry and materials (no dataset)",
            "config": workload_config(args.config, cfg, world),
            "e2e": {"value": e2e_ms / world if e2e_ms else None, "unit": "ms/solve", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": TRAFFIC_PER_ALGO_BYTE * bytes_order,
                         "kernel": "one exchange order: k_scatter_f32 + k_mix4 + k_add_e0_t launches", "peak_of": peak_kind,
                         "algorithmic_bytes": bytes_order, "ms_per_launch": ms_order,
                         "binding": "shared-memory bandwidth of k_scatter_f32 (roofline_smem); the order's HBM "
                                    "traffic is a byproduct"},
            "roofline_smem": smem,
            "cpu_baseline": cpu,
            "fp64_gpu": fp64,
            "sum_forms": sum_forms,
            "fwd_bwd": fwd_bwd,
            "configs": configs,
            "general_brdf": general,
            "batch": batch,
            "clocks": clk,
            "gpu_launches": int(launches),
            "exchange": {"algorithm": stats["algorithm"], "directed_pairs": n_pairs,
                         "source_groups": stats["source_groups"], "segments": stats["segments"],
                         "tiles": stats["tiles"], "ms_all_orders": float(np.mean(order_ms))},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------ per-config legs
def _gpu_solve_timed(cfg, precision, repeats=2):
    """Solve a config through the public API on the GPU: (ms per solve, mono histograms, radiosity)."""
    import torch
    from sparrowpy_gb300 import scenes
    c = scenes.config(cfg, precision=precision)
    r = c["radiosity"]
    st = torch.cuda.current_stream()
    ms = []
    for k in range(repeats + 1):  # the first solve warms up
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        solve(r, c, as_coords)
        e1.record(st)
        e1.synchronize()
        if k > 0:
            ms.append(e0.elapsed_time(e1))
    mono = r.collect_energy_receiver_mono(as_coords(c["receivers"])).time
    return float(np.mean(ms)), mono, r


def _triangle_leg(cfg):
    """The config's room with every patch cut into two triangles (FP32): ms per solve through the public API,
    against the quadrilateral room, and how the form factors were computed (triangles take the FP32 moment
    path; shared-vertex pairs the FP64 Nusselt analogue)."""
    import torch
    from sparrowpy_gb300 import DirectionalRadiosityFast, scenes
    c = scenes.config(cfg, precision="fp32")
    r = c["radiosity"]
    q = np.asarray(r._patches_points)
    tris = np.stack([q[:, [0, 1, 2]], q[:, [0, 2, 3]]], axis=1).reshape(-1, 3, 3)
    t = DirectionalRadiosityFast(r._walls_points, r._walls_normal, r._walls_up_vector, tris, tris.shape[0],
                                 np.repeat(np.asarray(r._patch_to_wall_ids), 2), frequencies=r._frequencies,
                                 air_attenuation=r._air_attenuation, precision="fp32")
    t._brdf = [np.array(b) for b in r._brdf]
    t._brdf_index = r._brdf_index.copy()
    t._brdf_incoming_directions = r._brdf_incoming_directions.copy()
    t._brdf_outgoing_directions = r._brdf_outgoing_directions.copy()
    del r
    st = torch.cuda.current_stream()
    ms = []
    for k in range(3):  # the first solve warms up
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        solve(t, c, as_coords)
        e1.record(st)
        e1.synchronize()
        if k > 0:
            ms.append(e0.elapsed_time(e1))
    method = t._bake["ff_method"].cpu().numpy()[: int(t._bake["n_vis"])]
    out = {"patches": int(t.n_patches), "fp32_ms_per_solve": float(np.mean(ms)),
           "exchange_ms": float(t.exchange_stats["order_ms"]),
           "form_factor_pairs": {"fp32_stokes": int((method == 0).sum()), "fp64_stokes": int((method == 1).sum()),
                                 "nusselt": int((method == 2).sum())}}
    del t
    torch.cuda.empty_cache()
    return out


def config_legs(cpu_shoebox_126=None):
    """shoebox_126 and shoebox_2016 at FP32 and FP64 on the GPU, with their errors and the FP64 energy check.

    shoebox_126 (126 patches) is also solved completely by the oracle on the host
    (cpu_shoebox_126: the result of cpu_full_solve_shoebox_126), which gives the error
    against the FP64 oracle and a measured CPU/GPU ratio; shoebox_2016 (2016 patches)
    is too large for a complete oracle solve, so its FP32 error is stated
    against the FP64 GPU solve (itself oracle-checked at 1e-10 on smaller
    scenes).
    """
    import torch
    out = {}
    for name in ("shoebox_126", "shoebox_2016"):
        leg = {}
        ms32, m32, r32 = _gpu_solve_timed(name, "fp32")
        eb32 = r32.energy_balance()
        del r32
        torch.cuda.empty_cache()
        ms64, m64, r64 = _gpu_solve_timed(name, "fp64", repeats=1)
        eb64 = r64.energy_balance()
        del r64
        torch.cuda.empty_cache()
        leg.update(fp32_ms_per_solve=ms32, fp64_ms_per_solve=ms64, fp64_over_fp32=ms64 / ms32,
                   receiver_rel_l2_fp32_vs_fp64_gpu=float(np.linalg.norm(m32 - m64) / np.linalg.norm(m64)),
                   energy_check={"fp32_max_rel_dev": float(eb32["rel_dev"].max()),
                                 "fp64_max_rel_dev": float(eb64["rel_dev"].max()),
                                 "check_ms": eb32["ms"],
                                 "meaning": "per-band FP64 sum of E_total against the time-free energy budget of "
                                            "the orders; nothing is delayed past this histogram"})
        if name == "shoebox_2016":
            leg["triangles"] = _triangle_leg(name)
        if name == "shoebox_126" and cpu_shoebox_126 is not None:
            cpu_ms, cores, desc, mono_ref = cpu_shoebox_126
            leg.update(receiver_rel_l2_fp32_vs_oracle=float(np.linalg.norm(m32 - mono_ref) / np.linalg.norm(mono_ref)),
                       receiver_rel_l2_fp64_vs_oracle=float(np.linalg.norm(m64 - mono_ref) / np.linalg.norm(mono_ref)),
                       cpu_measured={"ms": cpu_ms, "cores": cores, "sample": desc},
                       cpu_over_gpu_fp32=cpu_ms / ms32)
        out[name] = leg
    return out


# ------------------------------------------------------------ general BRDF
def general_brdf_leg(orders=50, dense_orders=5, patch_size=0.25):
    """A table without diffuse-plus-mirror structure on every wall: the 2016-patch shoebox's geometry and histogram.

    5 x 6 x 3 m shoebox at 0.25 m (2016 patches), one seeded random positive
    64 x 64 x 6 table (as create_from_directional_scattering tables are
    dense), T = 2000, FP32.  The general exchange (class scatter, then the
    receiver-side contraction of the 64 table rows) with the contraction on
    the tensor cores and on the CUDA cores, `orders` orders each, and the
    dense kernel (D FMAs per pair and bin) for `dense_orders` orders; per
    order ms from CUDA events around the order loop.
    """
    import torch
    from sparrowpy_gb300 import scenes
    from sparrowpy_gb300.brdf import hemisphere_directions
    from sparrowpy_gb300.coords import FrequencyData

    def room():
        r = scenes.shoebox(patch_size, n_dirs=64, n_bins=6, scattering=0.3, absorption=0.1, precision="fp32")
        rng = np.random.default_rng(9)
        dirs = hemisphere_directions(64)
        tab = rng.uniform(0.05, 0.25, size=(64, 64, 6)) / 8.0
        r.set_wall_brdf(np.arange(r.n_walls), FrequencyData(tab, np.asarray(r._frequencies, float)), dirs, dirs)
        return r

    out = {"workload": f"the 5 x 6 x 3 m shoebox at {patch_size} m patches, a seeded random positive 64 x 64 x 6 "
                       "BRDF table on every wall, 6 bands, T=2000, FP32"}
    monos = {}
    for name, algo, tc, k in (("general_tensor_cores", "general", True, orders),
                              ("general_cuda_cores", "general", False, orders),
                              ("dense", "dense", True, dense_orders)):
        r = room()
        r.tensor_cores = tc
        src = np.array([2.0, 2.0, 1.5])
        r.bake_geometry()
        r.init_source_energy(as_coords(src))
        for _ in range(2):  # the first call warms up
            r.calculate_energy_exchange(343.0, 1e-3, 2.0, k, recalculate=True, algorithm=algo)
        st = r.exchange_stats
        out[name] = {"orders": k, "ms_per_order": st["order_ms"] / k, "algorithm": st["algorithm"]}
        if st.get("scatter_ms", -1.0) >= 0 and st["algorithm"] != "dense":
            out[name]["scatter_ms_per_order"] = st["scatter_ms"] / k
            out[name]["contraction_ms_per_order"] = (st["order_ms"] - st["scatter_ms"]) / k
        if k == orders:
            monos[name] = r.collect_energy_receiver_mono(as_coords(np.array([[3.0, 4.0, 1.5]]))).time
        del r
        torch.cuda.empty_cache()
    a, b = monos["general_tensor_cores"], monos["general_cuda_cores"]
    out["receiver_rel_l2_tensor_vs_cuda_cores"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return out


# ------------------------------------------------------- forward + backward
def fwd_bwd_config4(steps=2, fd_params=64, seed=4, fp64_reference=True):
    """Energy-decay-loss gradient w.r.t. per-patch, per-band absorption and scattering.

    Timing: shoebox 5 x 6 x 3 m, 0.25 m patches, one wall per patch (2016
    patches), 6 bands, 64 directions, 1 ms x 2 s, order 50, 1 source, 1
    receiver; the target comes from a second seeded material set.  Times the
    FP32 forward solve (with checkpoints) and forward + backward with CUDA
    events.  References (fp64_reference):
      * the FP64 adjoint of the same room (FP64 forward, checkpoints and
        adjoint), against which every one of the 24,192 FP32 gradients is
        compared;
      * central differences (h = 1e-4) of the FP64 forward on `fd_params`
        seeded random parameters, on the same materials model over the
        126-patch shoebox (the 5 x 6 x 3 m room at 1 m patches, same
        bands, directions, histogram and order): 128 FP64 solves there take
        seconds, where the 2016-patch room's would take about 15 minutes.
    """
    import torch
    from sparrowpy_gb300.adjoint import DifferentiableExchange, as_source, energy_decay_loss, per_patch_room
    from sparrowpy_gb300.brdf import hemisphere_directions
    dirs = hemisphere_directions(64)
    src, rcv = np.array([2.0, 2.0, 1.5]), np.array([[3.0, 4.0, 1.5]])
    dev = "cuda"
    t = lambda x, g=False: torch.tensor(x, dtype=torch.float64, device=dev, requires_grad=g)
    st = torch.cuda.current_stream()

    def room(patch, precision):
        r = per_patch_room((5.0, 6.0, 3.0), patch, dirs, 6, precision=precision)
        return r, DifferentiableExchange(r, dirs, as_source(src), rcv, 343.0, 1e-3, 2.0, 50)

    def grads(solver, alpha0, scat0, target, n_steps):
        fwd_ms, both_ms = [], []
        for k in range(n_steps + 1):  # the first pass warms up
            a_t, s_t = t(alpha0, True), t(scat0, True)
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(st)
            loss = energy_decay_loss(solver(a_t, s_t), target)
            e1.record(st)
            loss.backward()
            e2.record(st)
            e2.synchronize()
            if k > 0 or n_steps == 0:
                fwd_ms.append(e0.elapsed_time(e1))
                both_ms.append(e0.elapsed_time(e2))
        return a_t.grad.cpu().numpy(), s_t.grad.cpu().numpy(), fwd_ms, both_ms

    rng = np.random.default_rng(seed)
    r, solver = room(0.25, "fp32")
    S = solver.n_slots
    alpha0, scat0 = rng.uniform(0.02, 0.6, (S, 6)), rng.uniform(0.1, 0.9, (S, 6))
    alpha_t, scat_t = rng.uniform(0.02, 0.6, (S, 6)), rng.uniform(0.1, 0.9, (S, 6))
    target = solver.forward_only(t(alpha_t), t(scat_t))
    ga, gs, fwd_ms, both_ms = grads(solver, alpha0, scat0, target, steps)
    out = {"workload": "shoebox 5x6x3 m, 0.25 m patches, one wall per patch: 2016 patches, 6 bands, 64 directions, "
                       "T=2000, order 50; loss = sum (log EDC - log EDC_target)^2",
           "params": int(ga.size + gs.size), "fwd_ms": float(np.mean(fwd_ms)), "fwd_bwd_ms": float(np.mean(both_ms)),
           "fwd_bwd_over_fwd": float(np.mean(both_ms) / np.mean(fwd_ms)), "checkpoint_every": solver.m}
    del solver, r
    torch.cuda.empty_cache()
    if fp64_reference:
        # the FP64 adjoint of the 2016-patch room would hold about 340 GB (FP64 checkpoints, exchange and adjoint
        # workspaces): the reference gradient runs on the same room at 0.5 m patches (504 patches, 6048 params)
        grad = {}
        for prec in ("fp32", "fp64"):
            rr, sv = room(0.5, prec)
            Sm = sv.n_slots
            rng_m = np.random.default_rng(seed + 7)
            a0, s0 = rng_m.uniform(0.02, 0.6, (Sm, 6)), rng_m.uniform(0.1, 0.9, (Sm, 6))
            tgt = sv.forward_only(t(rng_m.uniform(0.02, 0.6, (Sm, 6))), t(rng_m.uniform(0.1, 0.9, (Sm, 6))))
            grad[prec] = grads(sv, a0, s0, tgt, 0)
            del sv, rr
            torch.cuda.empty_cache()
        g32 = np.concatenate([grad["fp32"][0].ravel(), grad["fp32"][1].ravel()])
        g64 = np.concatenate([grad["fp64"][0].ravel(), grad["fp64"][1].ravel()])
        big = np.abs(g64) > 1e-3 * np.abs(g64).max()
        out["fp64_adjoint"] = {
            "workload": "the same room and loss at 0.5 m patches: 504 patches, 6048 parameters",
            "fp32_fwd_bwd_ms": float(grad["fp32"][3][0]), "fp64_fwd_bwd_ms": float(grad["fp64"][3][0]),
            "max_abs_err_over_max_grad": float(np.abs(g32 - g64).max() / np.abs(g64).max()),
            "rel_l2": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64)),
            "max_rel_err_where_grad_above_1e-3_max": float((np.abs(g32 - g64)[big] / np.abs(g64)[big]).max())}
    if fd_params > 0:
        out["fd_check"] = fd_check_shoebox_126_geometry(fd_params, seed=seed + 1)
    return out


def fd_check_shoebox_126_geometry(n_params, seed=5, h=1e-4):
    """FP32 and FP64 adjoint gradients against central differences of the FP64 forward (h = 1e-4).

    Per-patch materials over the 126-patch shoebox (5 x 6 x 3 m, 1 m
    patches), 6 bands, 64 directions, T = 2000, order 50; `n_params`
    seeded random (absorption or scattering, patch, band) entries.
    """
    import torch
    from sparrowpy_gb300.adjoint import DifferentiableExchange, as_source, energy_decay_loss, per_patch_room
    from sparrowpy_gb300.brdf import hemisphere_directions
    dirs = hemisphere_directions(64)
    src, rcv = np.array([2.0, 2.0, 1.5]), np.array([[3.0, 4.0, 1.5]])
    t = lambda x, g=False: torch.tensor(x, dtype=torch.float64, device="cuda", requires_grad=g)
    rng = np.random.default_rng(seed)
    solvers = {}
    for prec in ("fp32", "fp64"):
        r = per_patch_room((5.0, 6.0, 3.0), 1.0, dirs, 6, precision=prec)
        solvers[prec] = DifferentiableExchange(r, dirs, as_source(src), rcv, 343.0, 1e-3, 2.0, 50)
    S = solvers["fp64"].n_slots
    alpha0, scat0 = rng.uniform(0.02, 0.6, (S, 6)), rng.uniform(0.1, 0.9, (S, 6))
    target = solvers["fp64"].forward_only(t(rng.uniform(0.02, 0.6, (S, 6))), t(rng.uniform(0.1, 0.9, (S, 6))))
    g = {}
    for prec, sv in solvers.items():
        a_t, s_t = t(alpha0, True), t(scat0, True)
        energy_decay_loss(sv(a_t, s_t), target).backward()
        g[prec] = (a_t.grad.cpu().numpy(), s_t.grad.cpu().numpy())
    flat = rng.choice(2 * S * 6, size=n_params, replace=False)
    entries = []
    for q in flat:
        which, k = int(q >= S * 6), int(q % (S * 6))
        idx = np.unravel_index(k, (S, 6))
        vals = []
        for sign in (1, -1):
            a, s_ = alpha0.copy(), scat0.copy()
            (a if which == 0 else s_)[idx] += sign * h
            vals.append(float(energy_decay_loss(solvers["fp64"].forward_only(t(a), t(s_)), target)))
        fd = (vals[0] - vals[1]) / (2 * h)
        entries.append({"param": ["absorption", "scattering"][which], "index": [int(x) for x in idx],
                        "central_difference_fp64": fd, "adjoint_fp64": float(g["fp64"][which][idx]),
                        "adjoint_fp32": float(g["fp32"][which][idx])})
    fd = np.array([e["central_difference_fp64"] for e in entries])
    a64 = np.array([e["adjoint_fp64"] for e in entries])
    a32 = np.array([e["adjoint_fp32"] for e in entries])
    scale = np.abs(fd).max()
    return {"workload": "per-patch materials over the 126-patch shoebox (5x6x3 m, 1 m patches), 6 bands, "
                        "64 directions, T=2000, order 50", "h": h, "params": int(n_params),
            "max_rel_err_fp64_adjoint": float(np.max(np.abs(a64 - fd) / np.maximum(np.abs(fd), 1e-300))),
            "max_err_over_scale_fp64_adjoint": float(np.abs(a64 - fd).max() / scale),
            "max_err_over_scale_fp32_adjoint": float(np.abs(a32 - fd).max() / scale),
            "median_rel_err_fp32_adjoint": float(np.median(np.abs(a32 - fd) / np.maximum(np.abs(fd), 1e-300))),
            "entries": entries}


# ------------------------------------------------------------------- batch
def batch_rooms(n_rooms, seed=5, rank=0, world=1, compare_rooms=16, fp64_sample=4):
    """The batch of seeded shoebox rooms (dims U[3, 20] m, 0.5 m patches, 6 bands, 32 directions, T = 1000, order 30,
    1 source + 4 receivers each), each memory-sized wave's exchange orders in one persistent launch.

    Rank r of N takes rooms r, r + N, ...; the job's time is the slowest
    rank's sum of per-wave device times (bake and prepare, the persistent
    exchange launch, the collection; the tuner's probe launches excluded).
    Also, on rank 0: the first `compare_rooms` rooms solved one after
    another and batched (rooms/s of both), and the FP32 batched receiver
    histograms of the `fp64_sample` smallest rooms against their FP64 solves.
    """
    import torch
    from sparrowpy_gb300.batch import BatchTuner, shoebox_rooms, solve_rooms, solve_rooms_batched
    from sparrowpy_gb300.replicas import gather_in_order, max_over_ranks, shard
    rooms = shoebox_rooms(n_rooms, seed=seed)
    idx, mine = shard(rooms, rank, world)
    tuner = BatchTuner()
    monos, stats = solve_rooms_batched(mine, tuner=tuner) if mine else ([], {"waves": []})
    wave_ms = [w["bake_prepare_ms"] + w["exchange_and_collect_ms"] for w in stats["waves"]]
    total = max_over_ranks(float(np.sum(wave_ms)))
    patches = gather_in_order(n_rooms, idx, [p for w in stats["waves"] for p in w["patches"]])
    out = {"workload": f"{n_rooms} seeded shoebox rooms (dims U[3, 20] m, 0.5 m patches, 6 bands, 32 directions, "
                       f"T=1000, order 30, 4 receivers), dealt round-robin to {world} GPU(s); per GPU, waves of rooms "
                       "that fit in memory, each wave's exchange orders in one persistent launch or in the rooms' "
                       "own launches, whichever the autotuner measures faster (the mode is per wave)",
           "rooms": n_rooms, "patches_min": int(min(patches)), "patches_mean": float(np.mean(patches)),
           "patches_max": int(max(patches)), "total_ms": total, "rooms_per_s": float(n_rooms / (total * 1e-3)),
           "waves": [{k: w[k] for k in ("rooms", "bake_prepare_ms", "exchange_ms", "exchange_and_collect_ms",
                                        "items", "mode", "window_bins", "ctas_per_sm")} for w in stats["waves"]],
           "tuner_ms": stats.get("tuner")}
    if rank == 0 and compare_rooms > 0:
        sub = rooms[:compare_rooms]
        _, ms_seq, _ = solve_rooms(sub)
        _, st2 = solve_rooms_batched(sub, tuner=tuner)
        ms_b = sum(w["bake_prepare_ms"] + w["exchange_and_collect_ms"] for w in st2["waves"])
        out["compare"] = {"rooms": compare_rooms, "one_by_one_ms": float(np.sum(ms_seq)), "batched_ms": float(ms_b),
                          "speedup": float(np.sum(ms_seq) / ms_b)}
    if rank == 0 and fp64_sample > 0 and mine:
        sizes = [p for w in stats["waves"] for p in w["patches"]]
        pick = list(np.argsort(sizes)[:fp64_sample])
        errs = []
        for q in pick:
            m64, _, _ = solve_rooms([mine[q]], precision="fp64")
            errs.append(float(np.linalg.norm(monos[q] - m64[0]) / np.linalg.norm(m64[0])))
        out["fp64_sample"] = {"rooms": [int(i) for i in pick], "patches": [int(sizes[i]) for i in pick],
                              "receiver_rel_l2_fp32_vs_fp64": errs}
    torch.cuda.empty_cache()
    return out


# ----------------------------------------------------------- reference arm
def run_reference(args):
    """The reference loops on the host cores: the oracle's FP64 C++/OpenMP port, bounded samples per step."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from sparrowpy_gb300 import scenes
    from oracle import oracle as orc
    cfg = scenes.config(args.config, precision="fp64")
    if args.max_order is not None:
        cfg["max_order"] = args.max_order
    times, desc, cores = [], "", orc.num_threads()
    for k in range(args.warmup + args.steps):
        ms, cores, desc = cpu_baseline(cfg, rows_per_thread=1, exchange_rows=4)
        if k >= args.warmup:
            times.append(ms)
    v = float(np.mean(times))
    s126_ms, s126_cores, s126_desc, _ = cpu_full_solve_shoebox_126()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms/solve", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded street-canyon geometry and materials (no dataset)",
            "config": workload_config(args.config, cfg, world),
            "cpu_baseline": {"value": v, "unit": "ms/solve", "cores": cores, "kind": "port", "sample": desc,
                             "measured_shoebox_126": {"ms": s126_ms, "cores": s126_cores, "sample": s126_desc}},
            "e2e": {"value": v, "unit": "ms/solve", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.leg is not None:
        import torch
        torch.cuda.set_device(dist_env()[2])
        if a.leg == "general":
            k = a.max_order or 50
            leg = general_brdf_leg(orders=k, dense_orders=min(k, 5), patch_size=a.general_patch)
        else:
            leg = batch_rooms(a.batch_rooms, compare_rooms=0, fp64_sample=0)
        print(json.dumps({"metric": f"{a.leg} leg", a.leg: leg}), flush=True)
    elif a.fwd_bwd_only:
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps({"metric": "fwd+bwd ms", "fwd_bwd": fwd_bwd_config4(steps=a.steps)}), flush=True)
    elif a.impl == "reference":
        run_reference(a)
    else:
        run_gpu(a)
