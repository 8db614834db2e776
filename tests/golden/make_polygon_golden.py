"""Golden form factors and point factors of triangles and other convex polygons, from the sparrowpy reference.

Run in the build container (the reference imports as in make_golden.py).
The reference's universal form factor (universal.py:54-96), its Stokes and
Nusselt integrals (integration.py:38-289) and its point-to-patch factor
(integration.py:295-344) accept polygons of any vertex count; its own tests
only use quadrilaterals.  This script evaluates them on seeded triangles,
pentagons and hexagons in the relations the exchange meets:

* facing pairs at several distances (Stokes);
* pairs sharing an edge or a vertex at an angle (the Nusselt analogue: the
  triangle branch of the surface sampling for triangles, the
  parallelogram of the first and last sides for the other polygons);
* randomly placed pairs;
* triangles against quadrilaterals (Stokes and Nusselt with different
  vertex counts);
* point factors (source and receiver mode).

Output: tests/golden/polygons.npz.  Usage:
    python tests/golden/make_polygon_golden.py [--ref /path/to/sparrowpy]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import import_reference  # noqa: E402

MAXV = 8


def regular(nv, radius=1.0, phase=0.0):
    a = phase + 2 * np.pi * np.arange(nv) / nv
    return np.stack([radius * np.cos(a), radius * np.sin(a), np.zeros(nv)], axis=1)


def rotate(p, axis, angle):
    axis = np.asarray(axis, float) / np.linalg.norm(axis)
    k = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    r = np.eye(3) + np.sin(angle) * k + (1 - np.cos(angle)) * k @ k
    return p @ r.T


def normal(p):
    n = np.cross(p[1] - p[0], p[2] - p[0])
    return n / np.linalg.norm(n)


def pairs_to_compute(rng):
    out = []
    for nv in (3, 5, 6):
        base = regular(nv, 1.0, 0.3)
        for d in (0.4, 1.0, 2.5):  # facing, reversed winding so that the normals face each other
            out.append(("facing", base, base[::-1] + [0.2, -0.1, d]))
        # a second polygon hinged on the first one's side 0-1 at 90 and 60 degrees (shared edge)
        e0, e1 = base[0], base[1]
        for ang in (np.pi / 2, np.pi / 3):
            moved = rotate(base - e0, e1 - e0, ang) + e0
            out.append(("edge", base, moved[::-1]))
        # sharing vertex 0 only
        moved = rotate(base - base[0], [0.3, 1.0, 0.2], 1.1) + base[0]
        out.append(("vertex", base, moved))
        for _ in range(2):  # random placement
            p2 = rotate(regular(nv, rng.uniform(0.4, 1.2), rng.uniform(0, 1)), rng.normal(size=3), rng.uniform(0, 3))
            out.append(("random", base, p2 + rng.uniform(-1, 1, 3) + [0, 0, 2.0]))
    tri = np.array([[0.0, 0, 0], [1.0, 0, 0], [0.0, 0.8, 0]])
    quad = np.array([[0.0, 0, 0], [0.0, 0.9, 0], [0.0, 0.9, 1.1], [0.0, 0, 1.1]])
    out.append(("tri_quad_edge", tri, np.array([[0.0, 0, 0], [0.0, 0.8, 0], [0.0, 0.8, 1.0], [0.0, 0, 1.0]])))
    out.append(("quad_tri_vertex", quad, tri))
    out.append(("tri_quad_far", tri, quad + [2.0, 0.5, 0.0]))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('SPARROWPY_SRC'),
                    help='sparrowpy source tree (default: $SPARROWPY_SRC)')
    args = ap.parse_args()
    if not args.ref:
        ap.error('give --ref or set SPARROWPY_SRC')
    mods = import_reference(args.ref)
    geo, uni = mods['geo'], mods['uni']
    integ = sys.modules['sparrowpy.form_factor.integration']
    rng = np.random.default_rng(2024)
    cases = pairs_to_compute(rng)
    n = len(cases)
    pi = np.zeros((n, MAXV, 3))
    pj = np.zeros((n, MAXV, 3))
    nvi = np.zeros(n, np.int32)
    nvj = np.zeros(n, np.int32)
    ni = np.zeros((n, 3))
    nj = np.zeros((n, 3))
    area_i = np.zeros(n)
    value = np.zeros(n)
    nusselt = np.zeros(n, bool)
    kinds = []
    for k, (kind, a, b) in enumerate(cases):
        kinds.append(kind)
        nvi[k], nvj[k] = len(a), len(b)
        pi[k, :len(a)], pj[k, :len(b)] = a, b
        ni[k], nj[k] = normal(a), normal(b)
        area_i[k] = geo._polygon_area(a)
        nusselt[k] = bool(geo._coincidence_check(b, a))
        if nusselt[k]:
            value[k] = integ.nusselt_integration(patch_i=a, patch_i_normal=ni[k], patch_j=b, patch_j_normal=nj[k],
                                                 nsamples=64)
        else:
            value[k] = integ.stokes_integration(patch_i=a, patch_j=b, patch_i_area=area_i[k])
        if len(a) == len(b):  # the universal entry point gives the same number
            u = uni.universal_form_factor(a, ni[k], area_i[k], b, nj[k])
            assert u == value[k]
    # point factors
    polys = [regular(3, 0.7, 0.1), regular(5, 0.9, 0.2), np.array([[0.0, 0, 0], [1.2, 0, 0], [0.0, 0.7, 0]])]
    points = np.array([[0.1, 0.2, 1.0], [-0.4, 0.3, 0.5], [2.0, -1.0, 3.0]])
    pt_poly = np.zeros((len(polys) * len(points) * 2, MAXV, 3))
    pt_nv = np.zeros(pt_poly.shape[0], np.int32)
    pt_point = np.zeros((pt_poly.shape[0], 3))
    pt_mode = np.zeros(pt_poly.shape[0], np.int32)
    pt_value = np.zeros(pt_poly.shape[0])
    k = 0
    for poly in polys:
        for p in points:
            for mode, name in ((0, 'source'), (1, 'receiver')):
                pt_poly[k, :len(poly)] = poly
                pt_nv[k], pt_point[k], pt_mode[k] = len(poly), p, mode
                pt_value[k] = integ.pt_solution(point=p, patch_points=poly, mode=name)
                k += 1
    np.savez_compressed(os.path.join(HERE, 'polygons.npz'), pi=pi, pj=pj, nvi=nvi, nvj=nvj, ni=ni, nj=nj,
                        area_i=area_i, value=value, nusselt=nusselt, kinds=np.array(kinds),
                        pt_poly=pt_poly, pt_nv=pt_nv, pt_point=pt_point, pt_mode=pt_mode, pt_value=pt_value)
    print(f"{n} pairs ({int(nusselt.sum())} Nusselt), {k} point factors")


if __name__ == '__main__':
    main()
