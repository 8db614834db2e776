"""Golden values of the reference's form_factor package (sparrowpy/form_factor/kang.py and universal.py).

Runs, with the stub modules of make_golden.py standing in for pyfar, sofar,
deepdiff and matplotlib (numba absent: plain Python loops):
* kang.patch2patch_ff_kang on two rooms of axis-aligned patches (a 1 m cube
  at 0.5 m and a 3 x 2 x 2.5 m room at 0.5 m), every pair of patches on
  different walls, both directions;
* kang._source2patch_energy_kang from three source points (with and without
  air attenuation, two bands) and kang._patch2receiver_energy_kang for three
  receivers;
* universal._source2patch_energy_universal and
  universal._patch2receiver_energy_universal on the cube's patches, every
  patch visible.
Writes tests/golden/form_factor.npz.

Usage:  python tests/golden/make_form_factor_golden.py [--ref /path/to/sparrowpy]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from make_golden import import_reference  # noqa: E402

ROOMS = {"cube": ((1.0, 1.0, 1.0), 0.5), "room": ((3.0, 2.0, 2.5), 0.5)}
SOURCES = np.array([[0.3, 0.4, 0.6], [0.5, 0.5, 0.5], [0.7, 0.2, 0.35]])
RECEIVERS = np.array([[0.6, 0.3, 0.4], [0.25, 0.75, 0.5], [0.5, 0.5, 0.9]])
ATTENUATION = np.array([0.002, 0.01])


def room_patches(dims, size):
    from sparrowpy_gb300.geometry import process_patches, shoebox_room_stub
    walls = shoebox_room_stub(*dims)
    pts, normals, _, wall_of = process_patches(np.array([w.pts for w in walls]), np.array([w.normal for w in walls]),
                                               size)
    centers = pts.sum(axis=1) / pts.shape[1]
    sizes = np.abs((pts[:, 0] - pts[:, 1]) - (pts[:, 1] - pts[:, 2]))
    i, j = np.nonzero(wall_of[:, None] != wall_of[None, :])
    return pts, centers, normals, sizes, np.stack([i, j], axis=1).astype(np.int32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('SPARROWPY_SRC'),
                    help='sparrowpy source tree (default: $SPARROWPY_SRC)')
    args = ap.parse_args()
    if not args.ref:
        ap.error('give --ref or set SPARROWPY_SRC')
    import_reference(args.ref)
    import importlib
    kang = importlib.import_module('sparrowpy.form_factor.kang')
    uni = importlib.import_module('sparrowpy.form_factor.universal')
    out = {"sources": SOURCES, "receivers": RECEIVERS, "attenuation": ATTENUATION}
    for name, (dims, size) in ROOMS.items():
        pts, centers, normals, sizes, pairs = room_patches(dims, size)
        out[f"{name}_points"], out[f"{name}_centers"] = pts, centers
        out[f"{name}_normals"], out[f"{name}_sizes"], out[f"{name}_pairs"] = normals, sizes, pairs
        out[f"{name}_ff"] = kang.patch2patch_ff_kang(centers, normals, sizes, pairs)
        scale = np.array(dims) if name == "room" else np.ones(3)
        for k, s in enumerate(SOURCES * scale):
            e, d = kang._source2patch_energy_kang(s, centers, normals, ATTENUATION, sizes, 2)
            e0, _ = kang._source2patch_energy_kang(s, centers, normals, None, sizes, 2)
            out[f"{name}_src{k}_energy"], out[f"{name}_src{k}_distance"], out[f"{name}_src{k}_energy_noatt"] = e, d, e0
        for k, r in enumerate(RECEIVERS * scale):
            out[f"{name}_rcv{k}_factor"] = kang._patch2receiver_energy_kang(r - centers, normals)
    pts, centers = out["cube_points"], out["cube_centers"]
    vis = np.ones(centers.shape[0], dtype=bool)
    for k, s in enumerate(SOURCES):
        e, d = uni._source2patch_energy_universal(s, centers, pts, vis, ATTENUATION, 2)
        out[f"uni_src{k}_energy"], out[f"uni_src{k}_distance"] = e, d
    for k, r in enumerate(RECEIVERS):
        out[f"uni_rcv{k}_factor"] = uni._patch2receiver_energy_universal(r, pts, vis)
    np.savez_compressed(os.path.join(HERE, 'form_factor.npz'), **out)
    print({k: np.shape(v) for k, v in out.items() if 'src0' in k or 'ff' in k})


if __name__ == '__main__':
    main()
