"""Generate golden vectors from the sparrowpy reference (run in the build container).

The reference (sparrowpy 1.0.1) imports pyfar, sofar, deepdiff and
matplotlib, which are not installed; numba is absent too, so its hot-path
functions run as plain NumPy FP64.  This script inserts stub modules for the
missing packages (pyfar's Coordinates / FrequencyData / TimeData are
replaced by the light classes of sparrowpy_gb300.coords), imports the
reference module functions from the read-only source tree and calls them in
the order of DirectionalRadiosityFast's methods (RadiosityFast.py:369-752)
on four small scenes (the last with triangular patches).  Inputs (built with sparrowpy_gb300's host code) and
outputs are written to tests/golden/<scene>.npz.

Usage:  python tests/golden/make_golden.py [--ref /path/to/sparrowpy] [scene ...]
"""
import argparse
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from sparrowpy_gb300 import coords, scenes  # noqa: E402
from sparrowpy_gb300.brdf import create_from_scattering, hemisphere_directions, sph_gaussian  # noqa: E402
from oracle.scene import scene_from_radiosity  # noqa: E402


def import_reference(path):
    class _Any:
        def __init__(self, *a, **k):
            pass

    def stub(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    stub('pyfar', Coordinates=coords.Coordinates, FrequencyData=coords.FrequencyData, TimeData=coords.TimeData,
         Orientations=_Any)
    stub('pyfar.io')
    stub('sofar')
    stub('deepdiff', DeepDiff=_Any)
    mpl = stub('matplotlib')
    mpl.axes = stub('matplotlib.axes', Axes=_Any)
    mpl.pyplot = stub('matplotlib.pyplot')
    sys.path.insert(0, path)
    import importlib
    mods = dict(geo=importlib.import_module('sparrowpy.geometry'),
                uni=importlib.import_module('sparrowpy.form_factor.universal'),
                rf=importlib.import_module('sparrowpy.classes.RadiosityFast'),
                brdf=importlib.import_module('sparrowpy.brdf'))
    return mods


def cube_scene():
    from sparrowpy_gb300 import DirectionalRadiosityFast, shoebox_room_stub
    r = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(1, 1, 1), 0.5)
    return _cube_materials(r)


def tri_scene():
    """The cube's room with every 0.5 m patch cut into two triangles (48 patches), the cube's materials on 6
    seeded random directions (the symmetric cube with a symmetric direction set has exact ties in the
    outgoing-direction argmin, which rounding alone decides)."""
    from sparrowpy_gb300 import DirectionalRadiosityFast, shoebox_room_stub
    q = DirectionalRadiosityFast.from_polygon(shoebox_room_stub(1, 1, 1), 0.5)
    quads = np.asarray(q._patches_points)
    tris = np.stack([quads[:, [0, 1, 2]], quads[:, [0, 2, 3]]], axis=1).reshape(-1, 3, 3)
    ids = np.repeat(np.asarray(q._patch_to_wall_ids), 2)
    r = DirectionalRadiosityFast(q._walls_points, q._walls_normal, q._walls_up_vector, tris, tris.shape[0], ids)
    rng = np.random.default_rng(31)
    v = rng.normal(size=(6, 3))
    v[:, 2] = np.abs(v[:, 2]) + 0.2
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return _cube_materials(r, coords.Coordinates.from_cartesian(v, weights=np.full(6, 2 * np.pi / 6)))


def _cube_materials(r, dirs=None):
    from sparrowpy_gb300 import FrequencyData
    if dirs is None:
        g = sph_gaussian(sh_order=1)
        keep = g.z > 0
        dirs = coords.Coordinates.from_cartesian(g.cartesian[keep], weights=g.weights[keep])
    freqs = np.array([125., 250., 500., 1000.])
    brdf = create_from_scattering(dirs, dirs, FrequencyData(np.full(4, 0.5), freqs),
                                  FrequencyData(np.array([0.1, 0.15, 0.2, 0.3]), freqs))
    r.set_wall_brdf(np.arange(6), brdf, dirs, dirs)
    r.set_air_attenuation(FrequencyData(np.array([0.001, 0.002, 0.004, 0.008]), freqs))
    setup = dict(source=np.array([0.3, 0.4, 0.45]), receivers=np.array([[0.6, 0.55, 0.35], [0.25, 0.7, 0.8]]),
                 c=343.0, dt=5e-4, duration=0.1, max_order=6)
    return r, setup, (dirs, dirs, 0.5, np.array([0.1, 0.15, 0.2, 0.3]), freqs)


def shoebox_126_scene():
    c = scenes.config('shoebox_126')
    r = c.pop('radiosity')
    dirs = hemisphere_directions(16)
    return r, c, (dirs, dirs, 1.0, np.array([0.1]), np.array([63.0]))


def rot_scene():
    r, src, rcv = scenes.rotated_room()
    return r, dict(source=src, receivers=rcv, c=343.0, dt=1e-3, duration=0.15, max_order=4), None


SCENES = {'cube': cube_scene, 'shoebox_126': shoebox_126_scene, 'rot': rot_scene, 'tri': tri_scene}


def run_reference(mods, sc, setup, brdf_inputs):
    geo, uni, rf = mods['geo'], mods['uni'], mods['rf']
    out = {}
    pts = sc['patches_points']
    p2w = sc['patch_to_wall_ids']
    normals = sc['walls_normal'][p2w]
    ctr = geo._calculate_center(pts)
    area = geo._calculate_area(pts)
    out['centers'], out['areas'] = ctr, area
    t = time.time()
    V = geo._check_patch2patch_visibility(ctr, normals, pts)
    out['t_vis'] = time.time() - t
    n = pts.shape[0]
    # RadiosityFast.py:377-387
    n_comb = int(np.sum(V))
    vp = np.empty((n_comb, 2), dtype=np.int32)
    k = 0
    for i in range(n):
        for j in range(n):
            if V[i, j]:
                vp[k] = (i, j)
                k += 1
    t = time.time()
    F = uni.patch2patch_ff_universal(pts, normals, area, vp)
    out['t_ff'] = time.time() - t
    receivers_array = sc['dirs_out']
    sources_array = sc['dirs_in']
    scattering = sc['brdf']
    scattering_index = sc['brdf_index']
    # RadiosityFast.py:402-414
    p2o = receivers_array.shape[1] * np.ones((n, n), dtype=np.int64)
    for j in range(n):
        vis = np.where((V + V.T)[:, j])
        p2o[vis, j] = rf.get_scattering_data_receiver_index(
            pos_i=ctr[vis], pos_j=ctr[j], receivers=receivers_array, wall_id_i=p2w[vis])
    n_bins = scattering.shape[-1]
    att = sc['air_attenuation']
    fft = rf._form_factors_with_directivity_dim(V, F, n_bins, ctr, area, att, p2w, scattering, scattering_index,
                                                sources_array, receivers_array)
    out.update(V=V, visible_patches=vp, F=F, p2o=p2o, ff_tilde=fft)
    # init_source_energy (RadiosityFast.py:475-521)
    src = setup['source']
    svis = geo._check_point2patch_visibility(eval_point=src, patches_center=ctr, surf_points=sc['walls_points'],
                                             surf_normal=sc['walls_normal'])
    e0, d0 = uni._source2patch_energy_universal(src, ctr, pts, svis, att, n_bins)
    e0dir = rf._add_directional(e0, src, ctr, n_bins, p2w, sources_array, receivers_array, scattering,
                                scattering_index)
    out.update(svis=svis, e0=e0, d0=d0, e0dir=e0dir)
    # calculate_energy_exchange (RadiosityFast.py:533-564)
    c, dt = setup['c'], setup['dt']
    n_samples = int(setup['duration'] / dt)
    dij = np.empty((n, n))
    for i in range(n):
        for j in range(n):
            dij[i, j] = np.linalg.norm(ctr[i, :] - ctr[j, :])
    t = time.time()
    etot = rf._energy_exchange(n_samples, e0dir, d0, dij, fft, p2o, c, dt, setup['max_order'], vp)
    out['t_exchange'] = time.time() - t
    out['etot'] = etot
    # _collect_energy_patches (RadiosityFast.py:686-752) with propagation
    rcv = np.atleast_2d(setup['receivers'])
    hist = np.empty((rcv.shape[0], n, n_bins, n_samples))
    for i in range(rcv.shape[0]):
        rvis = geo._check_point2patch_visibility(eval_point=rcv[i], patches_center=ctr,
                                                 surf_points=sc['walls_points'], surf_normal=sc['walls_normal'])
        pre = uni._patch2receiver_energy_universal(rcv[i], pts, rvis)
        ridx = rf.get_scattering_data_receiver_index(ctr, rcv[i], receivers_array, p2w)
        E = np.empty((n, n_bins, n_samples))
        for k in range(n):
            E[k, :] = etot[k, int(ridx[k]), :] * pre[k]
        hist[i] = rf._collect_receiver_energy(E, np.linalg.norm(ctr - rcv[i], axis=1), c, dt, att)
    out['patchwise'] = hist
    out['mono'] = np.sum(hist, axis=1)
    # calculate_direct_sound (RadiosityFast.py:629-655)
    r_ = np.sqrt(np.sum((rcv - src) ** 2, axis=-1))
    ds = np.ones((rcv.shape[0], n_bins)) * (1 / (4 * np.pi * r_ ** 2))[:, None]
    for b in range(n_bins):
        ds[:, b] *= np.exp(-att[b] * r_)
    out['direct'] = ds
    out['direct_delay'] = np.array(r_ / c / dt, dtype=int)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('SPARROWPY_SRC'),
                    help='sparrowpy source tree (default: $SPARROWPY_SRC)')
    ap.add_argument('scenes', nargs='*', default=list(SCENES))
    args = ap.parse_args()
    if not args.ref:
        ap.error('give --ref or set SPARROWPY_SRC')
    mods = import_reference(args.ref)
    for name in args.scenes:
        r, setup, bi = SCENES[name]()
        sc = scene_from_radiosity(r)
        t0 = time.time()
        res = run_reference(mods, sc, setup, bi)
        print(f"{name}: N={r.n_patches} reference run {time.time() - t0:.1f} s "
              f"(vis {res['t_vis']:.1f} s, ff {res['t_ff']:.1f} s, exchange {res['t_exchange']:.1f} s)")
        save = dict(
            # inputs
            walls_points=sc['walls_points'], walls_normal=sc['walls_normal'],
            walls_up_vector=np.asarray(r._walls_up_vector), patches_points=sc['patches_points'],
            patch_to_wall_ids=sc['patch_to_wall_ids'], dirs_in=sc['dirs_in'], dirs_out=sc['dirs_out'],
            brdf=sc['brdf'], brdf_index=sc['brdf_index'], air_attenuation=sc['air_attenuation'],
            source=setup['source'], receivers=np.atleast_2d(setup['receivers']),
            acoustics=np.array([setup['c'], setup['dt'], setup['duration'], setup['max_order']]),
            # outputs
            centers=res['centers'], areas=res['areas'], V=res['V'], visible_patches=res['visible_patches'],
            ff_pairs=res['F'][res['visible_patches'][:, 0], res['visible_patches'][:, 1]],
            p2o=res['p2o'].astype(np.int16), svis=res['svis'], d0=res['d0'], e0=res['e0'], e0dir=res['e0dir'],
            mono=res['mono'], direct=res['direct'], direct_delay=res['direct_delay'],
        )
        n = r.n_patches
        if n <= 40:
            save['ff_tilde'] = res['ff_tilde']
            save['etot'] = res['etot']
            save['patchwise'] = res['patchwise']
        else:
            # size-limited: E_total summed over time plus full rows of a few patches
            rows = np.linspace(0, n - 1, 6).astype(int)
            save['etot_rows_index'] = rows
            save['etot_rows'] = res['etot'][rows]
            save['etot_time_sum'] = res['etot'].sum(axis=-1)
            vp = res['visible_patches']
            sel = vp[np.linspace(0, vp.shape[0] - 1, 64).astype(int)]
            save['ff_tilde_pairs'] = sel
            save['ff_tilde_sel'] = np.concatenate([res['ff_tilde'][sel[:, 0], sel[:, 1]][None],
                                                   res['ff_tilde'][sel[:, 1], sel[:, 0]][None]], axis=0)
        if bi is not None:
            dirs_in, dirs_out, s, alpha, freqs = bi
            ref_brdf = mods['brdf'].create_from_scattering(
                dirs_in, dirs_out, coords.FrequencyData(np.full(freqs.size, s), freqs),
                coords.FrequencyData(alpha, freqs))
            save['brdf_reference'] = ref_brdf.freq
            save['brdf_dirs'] = dirs_in.cartesian
            save['brdf_weights'] = dirs_in.weights
            save['brdf_params'] = np.concatenate([[s], alpha, freqs])
        np.savez_compressed(os.path.join(HERE, f'{name}.npz'), **save)


if __name__ == '__main__':
    main()
