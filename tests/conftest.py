"""Shared fixtures: golden vectors, scene injection, GPU gating."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built library")


def load_golden(name):
    path = os.path.join(GOLDEN, f"{name}.npz")
    if not os.path.exists(path):
        pytest.skip(f"golden fixture {name}.npz missing")
    with np.load(path, allow_pickle=False) as f:
        return {k: f[k] for k in f.files}


def scene_from_golden(g):
    """Oracle scene dict from the stored golden inputs."""
    att = g["air_attenuation"]
    return dict(patches_points=g["patches_points"], patch_to_wall_ids=g["patch_to_wall_ids"].astype(np.int64),
                walls_points=g["walls_points"], walls_normal=g["walls_normal"], dirs_in=g["dirs_in"],
                dirs_out=g["dirs_out"], brdf=g["brdf"], brdf_index=g["brdf_index"].astype(np.int64),
                air_attenuation=None if att.shape == () else att)


def radiosity_from_golden(g, precision="fp32"):
    """DirectionalRadiosityFast holding exactly the stored golden inputs."""
    from sparrowpy_gb300 import DirectionalRadiosityFast
    from sparrowpy_gb300.coords import Coordinates
    r = DirectionalRadiosityFast(g["walls_points"], g["walls_normal"], g["walls_up_vector"], g["patches_points"],
                                 g["patches_points"].shape[0], g["patch_to_wall_ids"], precision=precision)
    nb = g["brdf"].shape[-1]
    r._frequencies = np.arange(nb, dtype=float)
    r._brdf_incoming_directions = np.array([Coordinates.from_cartesian(d) for d in g["dirs_in"]] + [None],
                                           dtype=object)[:-1]
    r._brdf_outgoing_directions = np.array([Coordinates.from_cartesian(d) for d in g["dirs_out"]] + [None],
                                           dtype=object)[:-1]
    r._brdf = [np.array(b) for b in g["brdf"]]
    r._brdf_index = g["brdf_index"].astype(np.int64)
    r._air_attenuation = np.array(g["air_attenuation"], dtype=float)
    return r


def acoustics(g):
    c, dt, duration, k = g["acoustics"]
    return float(c), float(dt), float(duration), int(k)


def rel_l2(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(autouse=True)
def _skip_gpu_without_device(request):
    if request.node.get_closest_marker("gpu") is not None and not gpu_available():
        pytest.skip("no CUDA device")
