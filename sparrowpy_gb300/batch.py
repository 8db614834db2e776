"""Many independent rooms on one device.

A batch is a list of seeded shoebox rooms (dimensions, materials, source and
receivers drawn per room).

* `solve_rooms` runs the reference pipeline for each room in turn
  (bake_geometry, init_source_energy, calculate_energy_exchange,
  collect_energy_receiver_mono), releasing each room before the next.
* `solve_rooms_batched` bakes the rooms of a memory-sized wave (four host
  threads, one stream each), prepares each room's exchange (source energy,
  E_total and the pair plan in the room's workspace), then runs the
  exchange orders of the whole wave in one persistent launch
  (sp_exchange_batch: blocks pull scatter and mix pieces of every room from
  a device work queue, with bounded waits on the pieces they depend on), or
  in the rooms' own launches on their prepared plans, and collects each
  room's receivers.  The choice and the persistent launch's tile shape
  (scatter window of 1024 or 512 bins, blocks per SM) come from
  `BatchTuner`, which times the candidates on short runs of the first wave
  of each shape class and keeps the fastest.
"""
import concurrent.futures as cf
import ctypes
import itertools
import threading

import numpy as np
import torch

from . import _native as nat
from .brdf import create_from_scattering, hemisphere_directions
from .coords import Coordinates, FrequencyData
from .geometry import shoebox_room_stub
from .radiosity import DirectionalRadiosityFast, _ptr, _stream

OCTAVES6 = np.array([125.0, 250.0, 500.0, 1000.0, 2000.0, 4000.0])


def shoebox_rooms(n_rooms, seed=0, patch_size=0.5, dims_range=(3.0, 20.0), n_dirs=32, n_bins=6,
                  alpha_range=(0.02, 0.6), scattering=0.3, n_receivers=4):
    """Seeded room descriptions: dims per axis ~ U[dims_range] (whole patches), per-room, per-band
    absorption ~ U[alpha_range], one source and n_receivers receivers inside (0.5 m from the walls)."""
    rng = np.random.default_rng(seed)
    rooms = []
    for _ in range(n_rooms):
        dims = np.maximum(np.round(rng.uniform(*dims_range, size=3) / patch_size), 2) * patch_size
        alpha = rng.uniform(*alpha_range, size=n_bins)
        inner = lambda k: rng.uniform(0.5, dims - 0.5, size=(k, 3))
        rooms.append(dict(dims=dims, alpha=alpha, source=inner(1)[0], receivers=inner(n_receivers),
                          patch_size=patch_size, n_dirs=n_dirs, n_bins=n_bins, scattering=scattering))
    return rooms


def build_room(room, precision="fp32"):
    """DirectionalRadiosityFast of one room description (one material for all walls)."""
    walls = shoebox_room_stub(*room["dims"])
    r = DirectionalRadiosityFast.from_polygon(walls, room["patch_size"], precision=precision)
    freqs = OCTAVES6[:room["n_bins"]] if room["n_bins"] <= OCTAVES6.size else np.arange(1, room["n_bins"] + 1) * 1e3
    dirs = hemisphere_directions(room["n_dirs"])
    brdf = create_from_scattering(dirs, dirs, FrequencyData(np.full(freqs.size, room["scattering"]), freqs),
                                  FrequencyData(room["alpha"], freqs))
    r.set_wall_brdf(np.arange(r.n_walls), brdf, dirs, dirs)
    r.set_air_attenuation(FrequencyData(np.zeros(freqs.size), freqs))
    return r


def solve_rooms(rooms, speed_of_sound=343.0, etc_time_resolution=1e-3, etc_duration=1.0, max_reflection_order=30,
                precision="fp32", partial_sums=True):
    """Solve every room; returns (list of mono histograms (R, B, T) numpy, per-room device ms, patches).

    partial_sums: E_total as the last partial sum (DirectionalRadiosityFast.partial_sums)."""
    out, ms, patches = [], [], []
    st = torch.cuda.current_stream()
    for room in rooms:
        r = build_room(room, precision)
        r.partial_sums = partial_sums
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        r.bake_geometry()
        r.init_source_energy(Coordinates(*room["source"]))
        r.calculate_energy_exchange(speed_of_sound, etc_time_resolution, etc_duration, max_reflection_order)
        rc = room["receivers"]
        mono = r.collect_energy_receiver_mono(Coordinates(rc[:, 0], rc[:, 1], rc[:, 2])).time
        e1.record(st)
        e1.synchronize()
        out.append(mono)
        ms.append(e0.elapsed_time(e1))
        patches.append(r.n_patches)
        del r
    torch.cuda.empty_cache()
    return out, ms, patches


# ------------------------------------------------------------------ batched
_TAGS = itertools.count(1 << 40)  # plan tags of prepared rooms (process-wide, never 0)


class BatchTuner:
    """Tile choices of the persistent batched exchange, timed per shape class and kept.

    A shape class is (directions, bands, bins, size bucket of the wave's
    largest room).  Candidates: the persistent launch with scatter windows
    of 1024 and 512 bins and one to three blocks per SM, and ROOMS, the
    rooms' orders launched room after room on their prepared plans (the
    persistent launch's alternative where one room already fills the GPU).
    `choose` times each candidate (CUDA events) on `probe_orders` and on
    2 * probe_orders orders of the prepared wave, extrapolates each to the
    wave's order count (fixed cost plus cost per order: a short probe alone
    would favour the candidate with the smaller fixed cost), takes the
    fastest, and returns the cached choice for later waves of the class.
    """

    ROOMS = (0, 0)
    PERSISTENT = ((1024, 1), (1024, 2), (512, 1), (512, 2), (512, 3))
    CANDIDATES = PERSISTENT + (ROOMS,)

    def __init__(self, probe_orders=2):
        self.cache = {}
        self.timings = {}
        self.probe_orders = probe_orders

    @staticmethod
    def shape_class(nd, nb, nt, n_max):
        return (int(nd), int(nb), int(nt), int(np.ceil(np.log2(max(n_max, 1)))))

    def choose(self, key, run_probe, orders=None):
        """The cached choice of the shape class `key`, or the fastest candidate for `orders` orders (default:
        2 * probe_orders) by run_probe(candidate, k) -> ms."""
        if key not in self.cache:
            a = self.probe_orders
            b = 2 * a
            k = b if orders is None else max(int(orders), 1)
            times = {}
            for cand in self.CANDIDATES:
                ta, tb = run_probe(cand, a), run_probe(cand, b)
                times[cand] = ta + (k - a) * (tb - ta) / (b - a)
            self.timings[key] = times
            self.cache[key] = min(times, key=times.get)
        return self.cache[key]


_TUNER = BatchTuner()


def _room_bytes(n, nd, nb, nt, pairs, n_class):
    """Device bytes one prepared room holds (its exchange workspace, E_total and bake state)."""
    ws = nat.size("sp_energy_exchange_workspace", nat.SP_F32, nat.SP_EXCHANGE_STRUCTURED, n, nd, nb, nt, pairs, 1,
                  nd, n_class)
    return ws + n * nd * nb * nt * 4 + n * n * 9 + pairs * 60


class PreparedWave:
    """Rooms baked and prepared for one persistent batched exchange (all co-resident on the device).

    The room objects are built on the host first; `bake_prepare_ms` is the
    device time of the bakes, source energies and exchange preparations
    that follow (CUDA events), the part a one-by-one solve also spends.
    bake_threads rooms are baked at a time, each thread on its own stream.
    """

    def __init__(self, rooms, c, dt, nt, K, partial_sums=True, bake_threads=4):
        dev = torch.device("cuda", torch.cuda.current_device())
        st = torch.cuda.current_stream()
        self.c, self.dt, self.nt, self.K = c, dt, nt, K
        built = [build_room(room, "fp32") for room in rooms]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        # the rooms are baked and prepared by bake_threads host threads, each
        # on its own stream: a small room's bake is bound by launch latency
        # and host round trips, which the others' kernels then fill
        local = threading.local()
        streams = []
        lock = threading.Lock()

        def prepare(room, r):
            if not hasattr(local, "stream"):
                torch.cuda.set_device(dev)
                local.stream = torch.cuda.Stream(device=dev)
                local.stream.wait_event(start)
                with lock:
                    streams.append(local.stream)
            with torch.cuda.device(dev), torch.cuda.stream(local.stream):
                r.partial_sums = partial_sums
                r.bake_geometry()
                r.init_source_energy(Coordinates(*room["source"]))
                n, nd, nb = r._dev["e0dir"].shape
                etc = torch.empty((n, nd, nb, nt), dtype=torch.float32, device=dev)
                a = r._exchange_args(c, dt, nt, K, "auto", etc)
                a.prepare_only = 1
                a.plan_tag = next(_TAGS)
                n_class = 1 + nd if a.algorithm == nat.SP_EXCHANGE_SLOTWISE else a.n_groups * a.n_in_dirs
                wsz = nat.size("sp_energy_exchange_workspace", a.precision, a.algorithm, n, nd, nb, nt,
                               a.n_dir_pairs, a.n_slots, a.n_in_dirs, n_class)
                ws = torch.empty((wsz,), dtype=torch.uint8, device=dev)
                nat.call("sp_energy_exchange", ctypes.byref(a), _ptr(ws), wsz, _stream())  # the plan
            return r, a, (ws, wsz), etc

        start = torch.cuda.Event()
        start.record(st)
        workers = max(1, min(int(bake_threads), len(rooms)))
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            done = list(ex.map(prepare, rooms, built))
        for s_ in streams:
            st.wait_stream(s_)
        self.objs = [d[0] for d in done]
        self.args = [d[1] for d in done]
        self.wss = [d[2] for d in done]
        self.etcs = [d[3] for d in done]
        e1.record(st)
        e1.synchronize()
        self.bake_prepare_ms = e0.elapsed_time(e1)
        self.fresh = True  # E_0, E_total and the plans are in place for a launch
        self.rooms = (nat.BatchRoom * len(rooms))()
        for q, (a, (ws, wsz)) in enumerate(zip(self.args, self.wss)):
            self.rooms[q].args = ctypes.pointer(a)
            self.rooms[q].ws = ws.data_ptr()
            self.rooms[q].ws_bytes = wsz
        self.bsz = nat.size("sp_exchange_batch_workspace", len(rooms))
        self.bws = torch.empty((self.bsz,), dtype=torch.uint8, device=dev)
        # what sp_exchange_batch takes: FP32 rooms of one shape (directions, bands, bins) whose histogram
        # length is a multiple of 4 below 65536, in the structured, slot-wise or material exchange; other
        # waves run the rooms' own launches
        a0 = self.args[0]
        self.persistent_ok = nt % 4 == 0 and nt <= 65535 and all(
            a.precision == nat.SP_F32 and a.n_dir_pairs > 0 and
            a.algorithm in (nat.SP_EXCHANGE_STRUCTURED, nat.SP_EXCHANGE_SLOTWISE, nat.SP_EXCHANGE_MATERIAL) and
            (a.n_dirs, a.n_bins) == (a0.n_dirs, a0.n_bins) for a in self.args)

    def launch(self, choice, orders=None, wait_limit=0, force_timeout=False):
        """Run `orders` orders of every room in one launch (placing E_0 and E_total again, plans reused, unless
        the state prepared by the constructor is still unused).

        Returns (status, launch ms, work items); status is the C-ABI's.  The polls the items' dependency
        waits took are kept in `last_wait_polls`."""
        orders = self.K if orders is None else orders
        if tuple(choice) == BatchTuner.ROOMS:
            return self._launch_rooms(orders)
        if not self.fresh or orders != self.K:  # a launch consumed the prepared state: place it again
            for a, (ws, wsz) in zip(self.args, self.wss):
                a.max_order = orders
                nat.call("sp_energy_exchange", ctypes.byref(a), _ptr(ws), wsz, _stream())
        self.fresh = False
        ms = ctypes.c_float(-1.0)
        items = ctypes.c_longlong(0)
        b = nat.BatchArgs()
        b.n_rooms = len(self.args)
        b.rooms = self.rooms
        b.window_bins, b.ctas_per_sm = choice
        b.wait_limit = wait_limit
        b.force_timeout = 1 if force_timeout else 0
        b.exchange_ms = ctypes.pointer(ms)
        b.items = ctypes.pointer(items)
        polls = ctypes.c_longlong(0)
        b.wait_polls = ctypes.pointer(polls)
        rc = nat.lib().sp_exchange_batch(ctypes.byref(b), _ptr(self.bws), self.bsz, _stream())
        self.last_wait_polls = int(polls.value)
        return rc, float(ms.value), int(items.value)

    def _launch_rooms(self, orders):
        """The orders of each room by its own launches (sp_energy_exchange on the prepared plan, which places
        E_0 and E_total itself).  Returns (status, ms, 0) as launch does."""
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        rc = nat.SP_OK
        for a, (ws, wsz) in zip(self.args, self.wss):
            a.max_order = orders
            a.prepare_only = 0
            try:
                rc = nat.lib().sp_energy_exchange(ctypes.byref(a), _ptr(ws), wsz, _stream())
            finally:
                a.prepare_only = 1
            if rc != nat.SP_OK:
                break
        e1.record(st)
        e1.synchronize()
        self.fresh = False
        self.last_wait_polls = 0
        return rc, e0.elapsed_time(e1), 0

    def results(self, rooms):
        """Receiver histograms of each room after a full launch (collect_energy_receiver_mono)."""
        out = []
        for r, etc, room in zip(self.objs, self.etcs, rooms):
            r._dev["etc"] = etc
            r._etc_time_resolution, r._speed_of_sound, r._etc_duration = self.dt, self.c, self.nt * self.dt
            r._max_order = self.K
            rc = room["receivers"]
            out.append(r.collect_energy_receiver_mono(Coordinates(rc[:, 0], rc[:, 1], rc[:, 2])).time)
        return out


def solve_rooms_batched(rooms, speed_of_sound=343.0, etc_time_resolution=1e-3, etc_duration=1.0,
                        max_reflection_order=30, memory_fraction=0.6, tuner=None, force_choice=None,
                        partial_sums=True):
    """Solve every room, the exchange orders of each memory-sized wave in one persistent launch.

    Returns (list of mono histograms (R, B, T) numpy in room order, stats):
    stats holds per wave the rooms, their patch counts, the device ms of
    bake + prepare (after the room objects are built on the host, as
    solve_rooms times its rooms), of the batched exchange launch and of
    exchange + collection (a launch after the tuner's probes places E_0
    again first), the work items, the dependency-wait polls and the tile
    choice; plus the tuner's timings.  FP32; partial_sums as in solve_rooms.
    """
    tuner = tuner or _TUNER
    dev = torch.device("cuda", torch.cuda.current_device())
    st = torch.cuda.current_stream()
    c, dt = float(speed_of_sound), float(etc_time_resolution)
    nt = int(etc_duration / etc_time_resolution)
    K = int(max_reflection_order)
    free, _ = torch.cuda.mem_get_info(dev)
    budget = memory_fraction * (free + torch.cuda.memory_reserved(dev) - torch.cuda.memory_allocated(dev))
    out = [None] * len(rooms)
    waves = []
    i = 0
    while i < len(rooms):
        wave, used = [], 0.0
        while i < len(rooms):
            room = rooms[i]
            n_est = int(sum(2 * np.prod(np.round(np.delete(room["dims"], a) / room["patch_size"]))
                            for a in range(3)))
            need = _room_bytes(n_est, room["n_dirs"], room["n_bins"], nt, n_est * n_est, room["n_dirs"])
            if wave and used + need > budget:
                break
            wave.append(i)
            used += need
            i += 1
        waves.append(wave)
    stats = {"waves": []}
    for wave in waves:
        sub = [rooms[idx] for idx in wave]
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        pw = PreparedWave(sub, c, dt, nt, K, partial_sums)

        def probe(cand, k):
            rc, ms, _ = pw.launch(cand, min(k, K))
            if rc != nat.SP_OK:
                raise nat.NativeError("sp_exchange_batch", rc)
            return ms

        n_max = max(r.n_patches for r in pw.objs)
        nd, nb = pw.objs[0]._dev["e0dir"].shape[1:]
        key = BatchTuner.shape_class(nd, nb, nt, n_max)
        if force_choice:
            choice = force_choice
        elif not pw.persistent_ok:
            choice = BatchTuner.ROOMS
        else:
            choice = tuner.choose(key, probe, K)
        e[0].record(st)
        rc, ms_exchange, items = pw.launch(choice)
        if rc != nat.SP_OK:
            raise nat.NativeError("sp_exchange_batch", rc)
        monos = pw.results(sub)
        e[1].record(st)
        e[1].synchronize()
        for idx, mono in zip(wave, monos):
            out[idx] = mono
        stats["waves"].append({"rooms": len(wave), "patches": [int(r.n_patches) for r in pw.objs],
                               "bake_prepare_ms": pw.bake_prepare_ms, "exchange_ms": ms_exchange,
                               "exchange_and_collect_ms": e[0].elapsed_time(e[1]), "items": items,
                               "wait_polls": pw.last_wait_polls,
                               "mode": "rooms" if tuple(choice) == BatchTuner.ROOMS else "persistent",
                               "window_bins": choice[0], "ctas_per_sm": choice[1]})
        del pw
        torch.cuda.empty_cache()
    stats["tuner"] = {str(k): {f"{w}x{c_}": v for (w, c_), v in t.items()} for k, t in tuner.timings.items()}
    return out, stats
