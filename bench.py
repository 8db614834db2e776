#!/usr/bin/env python
"""Benchmark: milliseconds per solve (bake + exchange) of the street-canyon workload.

Workload (default ``--config cfg3``): two 100 x 20 m facades 15 m apart and a
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
os.environ.setdefault("PYTORCH_CUDA_ALLOC_CONF", "expandable_segments:True")

import numpy as np  # noqa: E402

METRIC = "ms/solve (bake+exchange) ~5.5k patches FP32 vs FP64 GPU; fwd+bwd ms; HBM GB/s"
PEAKS_FILE = os.path.join(HERE, "MEASURED_PEAKS.json")
# DRAM bytes moved per algorithmic byte by one exchange order (scatter + mix,
# averaged over a deferred and a pairing order), from the single-pass ncu
# capture summarised in profiles/exchange_street_canyon_small.md
TRAFFIC_PER_ALGO_BYTE = 1.20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--config", default="cfg3")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--max-order", type=int, default=None, help="override the workload's reflection order")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 GPU comparison solve")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-fwd-bwd", action="store_true", help="skip the gradient (forward + backward) leg")
    ap.add_argument("--batch-rooms", type=int, default=8, help="seeded shoebox rooms for the batch leg (0: skip)")
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


def algorithmic_bytes_per_order(n, d, b, t, pairs, n_slots, n_in, elem=4):
    """Bytes one exchange order must move at least.

    4 x N D B T histogram elements (read E_{k-1}, write E_k, read and write
    E_total) + 16 bytes per directed pair (F', delay, directions) + one read
    of the BRDF tables (S Din D B, FP32).
    """
    return 4.0 * elem * n * d * b * t + 16.0 * pairs + 4.0 * n_slots * n_in * d * b


def peak_hbm():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# -------------------------------------------------------------- CPU baseline
def cpu_baseline(cfg, rows_per_thread=1):
    """FP64 CPU restatement (oracle/) on bounded samples, extrapolated to one solve.

    GPU-free.  Samples, all on the same scene and its own pair lists:
      visibility - full rows of the visibility matrix at evenly spaced
                   patches (every pair against every blocker, as
                   geometry.py:750-797), scaled by N(N-1)/2 / pairs evaluated;
      form factors - the visible pairs (i < j) of those rows (universal.py),
                   scaled by the visible-pair count those rows imply;
      exchange   - one order of RadiosityFast.py:1121-1143 for the sampled
                   patches as destinations, their visible partners as sources
                   (true delays; source rows read from a 64-row buffer, the
                   cost does not depend on the values), times N / rows and
                   the number of orders.
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
    # one exchange order for the sampled rows as destinations
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
    t0 = time.perf_counter()
    orc.exchange_rows_sample(nd, nb, nt, prev, dst_off, src, p2o, delay, fprime, att, slot, s_in, sc["brdf"],
                             row_ids.astype(np.int32))
    t_order = (time.perf_counter() - t0) * n / rows.shape[0]
    total = t_vis + t_ff + cfg["max_order"] * t_order
    desc = (f"oracle C++/OpenMP FP64 on {threads} threads: visibility of {rows.shape[0]} full patch rows "
            f"({pairs_evaluated} pairs x {n} blockers), form factors of {pairs.shape[0]} of their visible pairs, "
            f"one exchange order for those {rows.shape[0]} destination patches ({m} incoming pairs); "
            f"extrapolated by pair/row counts to one solve: visibility {t_vis:.1f} s, form factors {t_ff:.1f} s, "
            f"{cfg['max_order']} orders x {t_order:.1f} s")
    return total * 1e3, threads, desc


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
    desc = {"cfg3": "street canyon: 100 x 20 m facades 15 m apart + 100 x 15 m ground, 1 m patches, 40 box occluders",
            "canyon_small": "street canyon: 30 x 20 m facades 15 m apart + ground, 1 m patches, 10 box occluders"}
    return {"workload": f"{desc.get(name, name)}; {r.n_patches} patches, {nb} bands, {nd} directions, "
                        f"{nt} x {cfg['dt'] * 1e3:g} ms bins, reflection order {cfg['max_order']}, 1 source",
            "name": name, "patches": r.n_patches, "bands": nb, "directions": nd, "bins": nt,
            "max_order": cfg["max_order"], "receivers": int(np.atleast_2d(cfg["receivers"]).shape[0]),
            "l2_policy": "inputs larger than L2 (each histogram array >= 1 GB), no flush",
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
        m32 = r.collect_energy_receiver_mono(as_coords(cfg["receivers"])).time
        err = float(np.linalg.norm(m32 - m64) / np.linalg.norm(m64))
        fp64 = {"ms_per_solve": float(np.mean(t64)), "fp64_over_fp32": float(np.mean(t64)) / ms_step,
                "exchange_ms_per_order": r64.exchange_stats["order_ms"] / max(stats["orders"], 1),
                "receiver_rel_l2_fp32_vs_fp64": err}
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
                         "kernel": "one exchange order: k_scatter_f32 + k_mix launches", "peak_of": peak_kind,
                         "algorithmic_bytes": bytes_order, "ms_per_launch": ms_order,
                         "binding": "shared-memory bandwidth of k_scatter_f32 (roofline_smem); the order's HBM "
                                    "traffic is a byproduct"},
            "roofline_smem": smem,
            "cpu_baseline": cpu,
            "fp64_gpu": fp64,
            "fwd_bwd": fwd_bwd,
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


# ------------------------------------------------------- forward + backward
def fwd_bwd_config4(steps=2, fd_params=2, seed=4):
    """Energy-decay-loss gradient w.r.t. per-patch, per-band absorption and scattering.

    Shoebox 5 x 6 x 3 m, 0.25 m patches, one wall per patch (2016 patches), 6
    bands, 64 directions, 1 ms x 2 s, order 50, 1 source, 1 receiver; the
    target comes from a second seeded material set.  Times the forward solve
    (with checkpoints) and forward + backward with CUDA events; checks the
    largest gradients against central differences of the FP32 forward.
    """
    import torch
    from sparrowpy_gb300.adjoint import DifferentiableExchange, as_source, energy_decay_loss, per_patch_room
    from sparrowpy_gb300.brdf import hemisphere_directions
    dirs = hemisphere_directions(64)
    r = per_patch_room((5.0, 6.0, 3.0), 0.25, dirs, 6)
    src, rcv = np.array([2.0, 2.0, 1.5]), np.array([[3.0, 4.0, 1.5]])
    solver = DifferentiableExchange(r, dirs, as_source(src), rcv, 343.0, 1e-3, 2.0, 50)
    rng = np.random.default_rng(seed)
    S = solver.n_slots
    dev = "cuda"
    t = lambda x, g=False: torch.tensor(x, dtype=torch.float64, device=dev, requires_grad=g)
    alpha0, scat0 = rng.uniform(0.02, 0.6, (S, 6)), rng.uniform(0.1, 0.9, (S, 6))
    target = solver.forward_only(t(rng.uniform(0.02, 0.6, (S, 6))), t(rng.uniform(0.1, 0.9, (S, 6))))
    st = torch.cuda.current_stream()
    fwd_ms, both_ms = [], []
    for k in range(steps + 1):  # first pass warms up
        a_t, s_t = t(alpha0, True), t(scat0, True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(st)
        loss = energy_decay_loss(solver(a_t, s_t), target)
        e1.record(st)
        loss.backward()
        e2.record(st)
        e2.synchronize()
        if k > 0:
            fwd_ms.append(e0.elapsed_time(e1))
            both_ms.append(e0.elapsed_time(e2))
    ga, gs = a_t.grad.cpu().numpy(), s_t.grad.cpu().numpy()
    fd = []
    h = 1e-3
    flat = np.abs(np.concatenate([ga.ravel(), gs.ravel()]))
    for q in np.argsort(flat)[::-1][:fd_params]:
        which, k = (0, q) if q < ga.size else (1, q - ga.size)
        idx = np.unravel_index(k, ga.shape)
        vals = []
        for sign in (1, -1):
            a, s_ = alpha0.copy(), scat0.copy()
            (a if which == 0 else s_)[idx] += sign * h
            vals.append(float(energy_decay_loss(solver.forward_only(t(a), t(s_)), target)))
        fdv = (vals[0] - vals[1]) / (2 * h)
        g = float((ga if which == 0 else gs)[idx])
        fd.append({"param": ["absorption", "scattering"][which], "index": [int(x) for x in idx], "adjoint": g,
                   "central_difference": fdv, "rel_err": abs(g - fdv) / max(abs(fdv), 1e-300)})
    out = {"workload": "shoebox 5x6x3 m, 0.25 m patches, one wall per patch: 2016 patches, 6 bands, 64 directions, "
                       "T=2000, order 50; loss = sum (log EDC - log EDC_target)^2",
           "params": int(ga.size + gs.size), "fwd_ms": float(np.mean(fwd_ms)), "fwd_bwd_ms": float(np.mean(both_ms)),
           "fwd_bwd_over_fwd": float(np.mean(both_ms) / np.mean(fwd_ms)), "checkpoint_every": solver.m,
           "fd_check_h": h, "fd_check": fd}
    del solver, r, target
    torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------------- batch
def batch_rooms(n_rooms, seed=5, rank=0, world=1):
    """Seeded shoebox rooms, dims U[3, 20] m, 0.5 m patches, 6 bands, 32 directions, 1 s, order 30,
    1 source + 4 receivers each.  Rank r of N solves rooms r, r + N, ... one after another; the job's
    time is the slowest rank's sum of per-room device times."""
    from sparrowpy_gb300.batch import shoebox_rooms, solve_rooms
    from sparrowpy_gb300.replicas import gather_in_order, max_over_ranks, shard
    rooms = shoebox_rooms(n_rooms, seed=seed)
    idx, mine = shard(rooms, rank, world)
    _, ms, patches = solve_rooms(mine) if mine else ([], [], [])
    total = max_over_ranks(float(np.sum(ms)))
    ms = gather_in_order(n_rooms, idx, [float(x) for x in ms])
    patches = gather_in_order(n_rooms, idx, [int(x) for x in patches])
    return {"workload": f"{n_rooms} seeded shoebox rooms (dims U[3, 20] m, 0.5 m patches, 6 bands, 32 directions, "
                        f"T=1000, order 30, 4 receivers), dealt round-robin to {world} GPU(s), one after another "
                        "on each",
            "rooms": n_rooms, "patches_min": int(min(patches)), "patches_mean": float(np.mean(patches)),
            "patches_max": int(max(patches)), "total_ms": total,
            "rooms_per_s": float(n_rooms / (total * 1e-3)), "ms_per_room": ms}


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
        ms, cores, desc = cpu_baseline(cfg, rows_per_thread=1)
        if k >= args.warmup:
            times.append(ms)
    v = float(np.mean(times))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ms/solve", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded street-canyon geometry and materials (no dataset)",
            "config": workload_config(args.config, cfg, world),
            "cpu_baseline": {"value": v, "unit": "ms/solve", "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": "ms/solve", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    a = parse()
    if a.fwd_bwd_only:
        import torch
        torch.cuda.set_device(dist_env()[2])
        print(json.dumps({"metric": "fwd+bwd ms", "fwd_bwd": fwd_bwd_config4(steps=a.steps, fd_params=0)}),
              flush=True)
    elif a.impl == "reference":
        run_reference(a)
    else:
        run_gpu(a)
