"""Seeded synthetic scenes of the benchmark and test workloads.

Every builder returns a configured DirectionalRadiosityFast plus the
acoustic setup (source, receivers, speed of sound, histogram resolution,
duration, maximum reflection order).  Scenes are deterministic for a seed.

* shoebox       - 5 x 6 x 3 m shoebox (sparrowpy/testing/stub_utils.py:5-48),
                  one BRDF for all walls or one wall per patch with per-patch,
                  per-band absorption (the reference keys BRDFs per wall,
                  RadiosityFast.py:804-816, so per-patch materials need one
                  wall per patch).
* street_canyon - two 100 x 20 m facades 15 m apart and a 100 x 15 m ground,
                  1 m patches, plus 40 seeded box occluders (5 patched faces
                  each) attached to the facades; one wall per patch.
* rotated_room  - a small room with a box inside, rotated and shifted to a
                  generic position (no coordinate-aligned planes).
"""
import numpy as np

from .brdf import create_from_scattering, hemisphere_directions, sph_gaussian
from .coords import Coordinates, FrequencyData
from .geometry import Polygon, process_patches, shoebox_room_stub
from .radiosity import DirectionalRadiosityFast

OCTAVES = np.array([63., 125., 250., 500., 1000., 2000., 4000., 8000.])


def _patch_polygons(walls, patch_size):
    """Split walls into one polygon per patch (keeps normals and up vectors)."""
    pts = np.array([w.pts for w in walls])
    nrm = np.array([w.normal for w in walls])
    patches, _, _, wall_ids = process_patches(pts, nrm, patch_size)
    return [Polygon(patches[k], walls[wall_ids[k]].up_vector, walls[wall_ids[k]].normal)
            for k in range(patches.shape[0])]


def _materials(r, dirs, freqs, scattering, absorption, per_wall_alpha=None):
    """One create_from_scattering BRDF per distinct absorption row."""
    sc = FrequencyData(np.full(freqs.size, scattering, dtype=float), freqs)
    if per_wall_alpha is None:
        brdf = create_from_scattering(dirs, dirs, sc, FrequencyData(np.asarray(absorption, float), freqs))
        r.set_wall_brdf(np.arange(r.n_walls), brdf, dirs, dirs)
    else:
        for w in range(r.n_walls):
            brdf = create_from_scattering(dirs, dirs, sc, FrequencyData(per_wall_alpha[w], freqs))
            r.set_wall_brdf([w], brdf, dirs, dirs)


def shoebox(patch_size=1.0, n_dirs=16, n_bins=1, scattering=1.0, absorption=0.1, per_patch=False,
            alpha_range=(0.02, 0.6), seed=0, dims=(5.0, 6.0, 3.0), air_attenuation=None, precision="fp32"):
    walls = shoebox_room_stub(*dims)
    if per_patch:
        walls = _patch_polygons(walls, patch_size)
    r = DirectionalRadiosityFast.from_polygon(walls, patch_size, precision=precision)
    freqs = OCTAVES[:n_bins] if n_bins <= OCTAVES.size else np.arange(1, n_bins + 1) * 100.0
    dirs = hemisphere_directions(n_dirs)
    if per_patch:
        rng = np.random.default_rng(seed)
        alpha = rng.uniform(alpha_range[0], alpha_range[1], size=(r.n_walls, freqs.size))
        _materials(r, dirs, freqs, scattering, None, per_wall_alpha=alpha)
    else:
        _materials(r, dirs, freqs, scattering, np.full(freqs.size, absorption))
    att = np.zeros(freqs.size) if air_attenuation is None else np.asarray(air_attenuation, float)
    r.set_air_attenuation(FrequencyData(att, freqs))
    return r


def _box_faces(x0, x1, y0, y1, z0, z1, skip_y0=True):
    """Outward faces of an axis-aligned box (the face on y = y0 omitted)."""
    faces = [
        Polygon([[x0, y1, z0], [x1, y1, z0], [x1, y1, z1], [x0, y1, z1]], [1, 0, 0], [0, 1, 0]),   # front
        Polygon([[x0, y0, z0], [x0, y0, z1], [x0, y1, z1], [x0, y1, z0]], [0, 0, 1], [-1, 0, 0]),  # left
        Polygon([[x1, y0, z0], [x1, y0, z1], [x1, y1, z1], [x1, y1, z0]], [0, 0, 1], [1, 0, 0]),   # right
        Polygon([[x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], [1, 0, 0], [0, 0, 1]),   # top
        Polygon([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0]], [1, 0, 0], [0, 0, -1]),  # bottom
    ]
    if not skip_y0:
        faces.append(Polygon([[x0, y0, z0], [x1, y0, z0], [x1, y0, z1], [x0, y0, z1]], [1, 0, 0], [0, -1, 0]))
    return faces


def street_canyon(n_boxes=40, patch_size=1.0, n_dirs=32, n_bins=8, scattering=0.3, alpha_range=(0.01, 0.3),
                  seed=0, length=100.0, height=20.0, width=15.0, precision="fp32"):
    """Street canyon: facades at y = 0 (normal +y) and y = width (normal -y), ground z = 0."""
    rng = np.random.default_rng(seed)
    L, H, Wd = length, height, width
    walls = [
        Polygon([[0, 0, 0], [L, 0, 0], [L, 0, H], [0, 0, H]], [1, 0, 0], [0, 1, 0]),
        Polygon([[0, Wd, 0], [L, Wd, 0], [L, Wd, H], [0, Wd, H]], [1, 0, 0], [0, -1, 0]),
        Polygon([[0, 0, 0], [L, 0, 0], [L, Wd, 0], [0, Wd, 0]], [1, 0, 0], [0, 0, 1]),
    ]
    occluders = []
    for k in range(n_boxes):
        sx, sy, sz = rng.uniform(1.0, 3.0, size=3)
        x0 = rng.uniform(1.0, L - 1.0 - sx)
        z0 = rng.uniform(1.0, H - 1.0 - sz)
        if k % 2 == 0:      # attached to the facade y = 0, protruding to +y
            faces = _box_faces(x0, x0 + sx, 0.0, sy, z0, z0 + sz)
        else:               # attached to the facade y = width, protruding to -y (mirror image)
            faces = [_mirror_y(f, Wd) for f in _box_faces(x0, x0 + sx, 0.0, sy, z0, z0 + sz)]
        occluders.extend(faces)
    all_walls = _patch_polygons(walls + occluders, patch_size)
    r = DirectionalRadiosityFast.from_polygon(all_walls, patch_size, precision=precision)
    freqs = OCTAVES[:n_bins]
    dirs = hemisphere_directions(n_dirs)
    alpha = rng.uniform(alpha_range[0], alpha_range[1], size=(r.n_walls, freqs.size))
    _materials(r, dirs, freqs, scattering, None, per_wall_alpha=alpha)
    r.set_air_attenuation(FrequencyData(np.zeros(freqs.size), freqs))
    return r


def _mirror_y(poly, width):
    """Mirror a polygon at the plane y = width / 2 (keeps outward normals)."""
    pts = poly.pts.copy()
    pts[:, 1] = width - pts[:, 1]
    n = poly.normal.copy()
    n[1] = -n[1]
    up = poly.up_vector.copy()
    up[1] = -up[1]
    pts = pts[::-1].copy()  # keep the winding consistent with the flipped normal
    return Polygon(pts, up, n)


def street_canyon_setup(seed=0, n_receivers=8, length=100.0, width=15.0):
    rng = np.random.default_rng(seed + 1000)
    src = np.array([rng.uniform(10, length - 10), rng.uniform(5.0, width - 5.0), 1.5])
    rcv = np.stack([rng.uniform(5, length - 5, n_receivers), rng.uniform(5.0, width - 5.0, n_receivers),
                    np.full(n_receivers, 1.5)], axis=1)
    return src, rcv


def rotation_matrix_xyz(ax, ay, az):
    cx, sx, cy, sy, cz, sz = np.cos(ax), np.sin(ax), np.cos(ay), np.sin(ay), np.cos(az), np.sin(az)
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return rz @ ry @ rx


ROT = rotation_matrix_xyz(0.3, 0.7, 1.1)
SHIFT = np.array([0.37, -1.21, 0.53])


def rotated_room(patch_size=0.5, n_dirs=8, n_bins=2, seed=3, precision="fp32", dense_box=True):
    """Room 3 x 2 x 2 m with a 0.6 m box on the floor, rotated to a generic pose.

    Room walls: diffuse-plus-mirror BRDF (s = 0.3); box faces: a seeded
    positive BRDF table without that structure when ``dense_box``.
    """
    room = shoebox_room_stub(3.0, 2.0, 2.0)
    # box corners off the patch grid: no centre-to-centre segment passes
    # exactly through a box edge (generic position)
    box = _box_faces(1.2113, 1.8187, 0.7071, 1.3091, 0.0, 0.6133, skip_y0=False)
    box = [f for f in box if f.normal[2] != -1]  # no face on the floor
    walls = room + box
    wp = np.array([w.pts for w in walls])
    wn = np.array([w.normal for w in walls])
    wu = np.array([w.up_vector for w in walls])
    pp, _, n, p2w = process_patches(wp, wn, patch_size)
    rot = lambda a: a @ ROT.T
    r = DirectionalRadiosityFast(rot(wp) + SHIFT, rot(wn), rot(wu), rot(pp) + SHIFT, n, p2w, precision=precision)
    freqs = OCTAVES[3:3 + n_bins]
    # seeded jitter of the direction set: a ring of equal colatitudes is
    # equidistant to a vector along the wall normal (an exact argmin tie)
    rng_d = np.random.default_rng(seed + 100)
    base = hemisphere_directions(n_dirs)
    col = np.clip(base.colatitude + rng_d.uniform(-0.08, 0.08, base.csize), 0.05, np.pi / 2 - 0.05)
    az = base.azimuth + rng_d.uniform(-0.08, 0.08, base.csize)
    dirs = Coordinates.from_spherical_colatitude(az, col, 1.0, weights=base.weights)
    brdf = create_from_scattering(dirs, dirs, FrequencyData(np.full(n_bins, 0.3), freqs),
                                  FrequencyData(np.linspace(0.1, 0.2, n_bins), freqs))
    r.set_wall_brdf(np.arange(6), brdf, dirs, dirs)
    if dense_box:
        rng = np.random.default_rng(seed)
        tab = rng.uniform(0.05, 0.3, size=(n_dirs, n_dirs, n_bins))
        r.set_wall_brdf(np.arange(6, r.n_walls), FrequencyData(tab, freqs), dirs, dirs)
    else:
        r.set_wall_brdf(np.arange(6, r.n_walls), brdf, dirs, dirs)
    r.set_air_attenuation(FrequencyData(np.linspace(0.001, 0.004, n_bins), freqs))
    src = np.array([0.6, 0.5, 1.3]) @ ROT.T + SHIFT
    rcv = np.array([[2.4, 1.5, 0.9], [0.5, 1.6, 1.6]]) @ ROT.T + SHIFT
    return r, src, rcv


# Workload table: name -> builder kwargs and acoustic setup
def config(name, precision="fp32"):
    if name == "shoebox_126":
        r = shoebox(1.0, n_dirs=16, n_bins=1, scattering=1.0, absorption=0.1, precision=precision)
        return dict(radiosity=r, source=np.array([2.0, 2.0, 1.5]), receivers=np.array([[3.0, 4.0, 1.5]]),
                    c=343.0, dt=1e-3, duration=1.0, max_order=20)
    if name == "shoebox_2016":
        r = shoebox(0.25, n_dirs=64, n_bins=6, scattering=0.3, per_patch=True, alpha_range=(0.02, 0.6), seed=2,
                    precision=precision)
        return dict(radiosity=r, source=np.array([2.0, 2.0, 1.5]), receivers=np.array([[3.0, 4.0, 1.5]]),
                    c=343.0, dt=1e-3, duration=2.0, max_order=50)
    if name == "street_canyon_5939":
        r = street_canyon(seed=3, precision=precision)
        src, rcv = street_canyon_setup(seed=3)
        return dict(radiosity=r, source=src, receivers=rcv, c=343.0, dt=1e-3, duration=2.0, max_order=50)
    if name == "street_canyon_1759":
        # the street canyon at 30 m length, 10 occluders and 2 bands (same
        # directions, patch size and histogram length): a profiling case
        # whose histograms stay near 1 GB each
        r = street_canyon(n_boxes=10, n_bins=2, seed=3, length=30.0, precision=precision)
        src, rcv = street_canyon_setup(seed=3, length=30.0)
        return dict(radiosity=r, source=src, receivers=rcv, c=343.0, dt=1e-3, duration=2.0, max_order=50)
    raise ValueError(name)

