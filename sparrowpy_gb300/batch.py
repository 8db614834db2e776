"""Many independent rooms through the solver, one after another on one device.

A batch is a list of seeded shoebox rooms (dimensions, materials, source and
receivers drawn per room).  `solve_rooms` runs the reference pipeline for
each (bake_geometry, init_source_energy, calculate_energy_exchange,
collect_energy_receiver_mono) and returns the receiver histograms with the
device time per room.  Rooms are not co-resident: each room's histograms and
workspace are released before the next room, so the batch needs only the
memory of its largest room.
"""
import numpy as np
import torch

from .brdf import create_from_scattering, hemisphere_directions
from .coords import Coordinates, FrequencyData
from .geometry import shoebox_room_stub
from .radiosity import DirectionalRadiosityFast

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
                precision="fp32"):
    """Solve every room; returns (list of mono histograms (R, B, T) numpy, per-room device ms, patches)."""
    out, ms, patches = [], [], []
    st = torch.cuda.current_stream()
    for room in rooms:
        r = build_room(room, precision)
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
