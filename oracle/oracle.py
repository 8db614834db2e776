"""FP64 CPU oracle of the directional fast-radiosity path (TEST INFRASTRUCTURE).

Restates the reference pipeline of sparrowpy 1.0.1
(sparrowpy/classes/RadiosityFast.py:369-752) on plain arrays, calling the
C++ restatement of its numba loops in oracle.cpp.  Used only by the tests,
the smoke check and the CPU-baseline leg of the benchmark, to check against;
the product (sparrowpy_gb300) never imports it.

A scene is a dict of numpy arrays:
  patches_points (N, nv, 3) with 3 <= nv <= 8, patch_to_wall_ids (N,), walls_points (W, nw, 3),
  walls_normal (W, 3), dirs_in (W, Din, 3), dirs_out (W, Dout, 3),
  brdf (S, Din, Dout, B) (already times pi), brdf_index (W,),
  air_attenuation (B,) or None.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None
_P = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        h = ctypes.CDLL(path)
        h.orc_stokes.restype = ctypes.c_double
        h.orc_nusselt.restype = ctypes.c_double
        h.orc_pt_solution.restype = ctypes.c_double
        _lib = h
    return _lib


def set_threads(n):
    lib().orc_set_num_threads(int(n))


def num_threads():
    return int(lib().orc_num_threads())


def _p(a):
    return a.ctypes.data_as(_P)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# ------------------------------------------------------------------ geometry
def centers(points):
    """geometry.py:412-413."""
    return np.sum(points, axis=-2) / points.shape[-2]


def areas(points):
    """geometry.py:420-448."""
    out = np.zeros(points.shape[0])
    for i in range(points.shape[0]):
        a = 0.0
        for t in range(points.shape[1] - 2):
            a += .5 * np.linalg.norm(np.cross(points[i, t + 1] - points[i, 0], points[i, t + 2] - points[i, 0]))
        out[i] = a
    return out


def patch_visibility(ctr, normals, points):
    """geometry.py:750-797 -> (N, N) bool, upper triangle."""
    n = ctr.shape[0]
    vis = np.zeros((n, n), dtype=np.uint8)
    ctr, normals, points = _c(ctr, float), _c(normals, float), _c(points, float)
    lib().orc_patch_visibility(n, points.shape[1], _p(ctr), _p(normals), _p(points), _p(vis))
    return vis.astype(bool)


def point_visibility(point, ctr, surf_points, surf_normals):
    """geometry.py:799-839 -> (N,) bool."""
    n = ctr.shape[0]
    out = np.zeros(n, dtype=np.uint8)
    point = _c(point, float)
    ctr, sp, sn = _c(ctr, float), _c(surf_points, float), _c(surf_normals, float)
    lib().orc_point_visibility(_p(point), n, _p(ctr), sp.shape[0], sp.shape[1], _p(sp), _p(sn), _p(out))
    return out.astype(bool)


def visible_pairs(vis):
    """RadiosityFast.py:377-387 (row-major list of (i, j), i < j)."""
    i, j = np.nonzero(vis)
    return np.stack([i, j], axis=1).astype(np.int32)


def form_factors(points, normals, area, pairs):
    """universal.py:12-52 -> values per listed pair."""
    pairs = _c(pairs, np.int32)
    out = np.zeros(pairs.shape[0])
    points, normals, area = _c(points, float), _c(normals, float), _c(area, float)
    rc = lib().orc_form_factors(pairs.shape[0], _p(pairs), _p(points), points.shape[1], _p(normals), _p(area),
                                _p(out))
    if rc != 0:
        raise ValueError("patches need 3 to 8 vertices")
    return out


def stokes(pi, pj, area_i):
    pi, pj = _c(pi, float), _c(pj, float)
    return lib().orc_stokes(_p(pi), pi.shape[0], _p(pj), pj.shape[0], ctypes.c_double(area_i))


def nusselt(pi, pj, ni, nj, nsamples=64):
    pi, pj = _c(pi, float), _c(pj, float)
    return lib().orc_nusselt(_p(pi), pi.shape[0], _p(pj), pj.shape[0], _p(_c(ni, float)), _p(_c(nj, float)),
                             nsamples)


def pt_solution(point, patch, mode="source"):
    return lib().orc_pt_solution(_p(_c(point, float)), _p(_c(patch, float)), patch.shape[0],
                                 1 if mode == "receiver" else 0)


def nearest_dirs(from_idx, to_idx, ctr, wall_of_pair, dirs):
    """argmin over dirs[wall_of_pair[p]] of |d - unit(c_to - c_from)|^2 (RadiosityFast.py:1277-1312)."""
    from_idx, to_idx = _c(from_idx, np.int32), _c(to_idx, np.int32)
    out = np.zeros(from_idx.shape[0], dtype=np.int32)
    ctr, wall_of, dirs = _c(ctr, float), _c(wall_of_pair, np.int64), _c(dirs, float)
    lib().orc_nearest_dirs(from_idx.shape[0], _p(from_idx), _p(to_idx), _p(ctr), _p(wall_of), _p(dirs),
                           dirs.shape[1], _p(out))
    return out


def point_dirs(point, ctr, wall_of, dirs):
    out = np.zeros(ctr.shape[0], dtype=np.int32)
    point, ctr, wall_of, dirs = _c(point, float), _c(ctr, float), _c(wall_of, np.int64), _c(dirs, float)
    lib().orc_point_dirs(_p(point), ctr.shape[0], _p(ctr), _p(wall_of), _p(dirs), dirs.shape[1], _p(out))
    return out


# --------------------------------------------------------------- pipeline
def bake(scene):
    """bake_geometry (RadiosityFast.py:369-433) on arrays."""
    pts = scene["patches_points"]
    wall_of = np.asarray(scene["patch_to_wall_ids"], dtype=np.int64)
    normals = scene["walls_normal"][wall_of]
    ctr = centers(pts)
    area = areas(pts)
    vis = patch_visibility(ctr, normals, pts)
    pairs = visible_pairs(vis)
    ff = form_factors(pts, normals, area, pairs)
    n = pts.shape[0]
    F = np.zeros((n, n))
    F[pairs[:, 0], pairs[:, 1]] = ff
    # directed pairs in the reference loop order (RadiosityFast.py:1124-1131)
    src = np.empty(2 * pairs.shape[0], dtype=np.int32)
    dst = np.empty_like(src)
    src[0::2], dst[0::2] = pairs[:, 0], pairs[:, 1]
    src[1::2], dst[1::2] = pairs[:, 1], pairs[:, 0]
    has_brdf = scene.get("dirs_in") is not None
    if has_brdf:
        # p2o: wall of the sender toward unit(c_dst - c_src) (RadiosityFast.py:402-414)
        p2o = nearest_dirs(src, dst, ctr, wall_of[src], scene["dirs_out"])
        # BRDF row: wall of the sender, unit(c_src - c_dst) (RadiosityFast.py:1264-1268)
        s_in = nearest_dirs(dst, src, ctr, wall_of[src], scene["dirs_in"])
    else:
        p2o = np.zeros_like(src)
        s_in = np.zeros_like(src)
    diff = ctr[src] - ctr[dst]
    dist = np.array([np.linalg.norm(v) for v in diff])
    unit = diff / dist[:, None]
    unit_len = np.array([np.linalg.norm(v) for v in unit])
    fprime = np.where(src < dst, F[src, dst], F[dst, src] * area[dst] / area[src])
    p2o_dense = np.full((n, n), scene["dirs_out"].shape[1] if has_brdf else 0, dtype=np.int64)
    if has_brdf:
        p2o_dense[src, dst] = p2o
    return dict(centers=ctr, areas=area, normals=normals, vis=vis, pairs=pairs, ff=ff, F=F, src=src, dst=dst,
                p2o=p2o, s_in=s_in, dist=dist, unit_len=unit_len, fprime=fprime, p2o_dense=p2o_dense,
                has_brdf=has_brdf)


def pair_att(scene, bk):
    att = scene.get("air_attenuation")
    nb = scene["brdf"].shape[-1] if bk["has_brdf"] else (1 if att is None else att.size)
    if att is None:
        return np.ones((bk["src"].size, nb))
    return np.exp(-np.asarray(att)[None, :] * bk["unit_len"][:, None])


def form_factors_tilde(scene, bk):
    """RadiosityFast.py:1234-1272 (dense; small scenes only)."""
    n = bk["centers"].shape[0]
    att = pair_att(scene, bk)
    if bk["has_brdf"]:
        slot = np.asarray(scene["brdf_index"])[np.asarray(scene["patch_to_wall_ids"])[bk["src"]]]
        rows = scene["brdf"][slot, bk["s_in"]]  # (P, D, B)
    else:
        rows = np.ones((bk["src"].size, 1, att.shape[1]))
    out = np.zeros((n, n, rows.shape[1], rows.shape[2]))
    out[bk["src"], bk["dst"]] = (bk["fprime"][:, None, None] * att[:, None, :]) * rows
    return out


def init_source(scene, bk, src_pos):
    """init_source_energy (RadiosityFast.py:436-522) -> E0dir (N, D, B), d0 (N,), vis (N,)."""
    pts = scene["patches_points"]
    ctr = bk["centers"]
    wall_of = np.asarray(scene["patch_to_wall_ids"], dtype=np.int64)
    svis = point_visibility(src_pos, ctr, scene["walls_points"], scene["walls_normal"])
    att = scene["air_attenuation"]
    nb = scene["brdf"].shape[-1]
    e0 = np.zeros((ctr.shape[0], nb))
    d0 = np.zeros(ctr.shape[0])
    for j in range(ctr.shape[0]):
        if svis[j]:
            d0[j] = np.linalg.norm(src_pos - ctr[j])
            e0[j] = np.exp(-att * d0[j]) * pt_solution(src_pos, pts[j], "source")
    sidx = point_dirs(src_pos, ctr, wall_of, scene["dirs_in"])
    slot = np.asarray(scene["brdf_index"])[wall_of]
    e0dir = e0[:, None, :] * scene["brdf"][slot, sidx]
    return e0dir, d0, svis


def exchange(scene, bk, e0dir, d0, c, dt, n_samples, max_order):
    """_energy_exchange (RadiosityFast.py:1073-1145) -> E_total (N, D, B, T) FP64."""
    n, nd, nb = e0dir.shape
    etot = np.zeros((n, nd, nb, n_samples))
    delay0 = np.array([int(x / c / dt) for x in d0], dtype=np.int64)
    delay = np.array([int(x / c / dt) for x in bk["dist"]], dtype=np.int64)
    att = pair_att(scene, bk)
    if bk["has_brdf"]:
        slot = np.asarray(scene["brdf_index"])[np.asarray(scene["patch_to_wall_ids"])[bk["src"]]].astype(np.int32)
        brdf = scene["brdf"]
        s_in = bk["s_in"]
        p2o = bk["p2o"]
    else:
        slot = np.zeros(bk["src"].size, dtype=np.int32)
        brdf = np.ones((1, 1, 1, nb))
        s_in = np.zeros(bk["src"].size, dtype=np.int32)
        p2o = np.zeros(bk["src"].size, dtype=np.int32)
    args = [_c(e0dir, float), _c(delay0, np.int64), _c(bk["src"], np.int32), _c(bk["dst"], np.int32),
            _c(p2o, np.int32), _c(delay, np.int64), _c(bk["fprime"], float), _c(att, float), _c(slot, np.int32),
            _c(s_in, np.int32), _c(brdf, float)]
    rc = lib().orc_exchange(n, nd, nb, n_samples, max_order, _p(args[0]), _p(args[1]), int(bk["src"].size),
                            _p(args[2]), _p(args[3]), _p(args[4]), _p(args[5]), _p(args[6]), _p(args[7]),
                            _p(args[8]), _p(args[9]), _p(args[10]), brdf.shape[1], _p(etot))
    if rc != 0:
        raise IndexError("source delay outside the histogram")
    return etot


def collect(scene, bk, etot, receivers, c, dt, patchwise=False):
    """_collect_energy_patches (RadiosityFast.py:686-752) -> (R, B, T) or (R, N, B, T)."""
    receivers = np.atleast_2d(receivers)
    n, nd, nb, nt = etot.shape
    wall_of = np.asarray(scene["patch_to_wall_ids"], dtype=np.int64)
    ctr = bk["centers"]
    att = scene["air_attenuation"]
    out = np.zeros((receivers.shape[0], n, nb, nt)) if patchwise else np.zeros((receivers.shape[0], nb, nt))
    e = _c(etot, float)
    for r, rp in enumerate(receivers):
        rvis = point_visibility(rp, ctr, scene["walls_points"], scene["walls_normal"])
        rfac = np.zeros(n)
        for k in range(n):
            if rvis[k]:
                rfac[k] = pt_solution(rp, scene["patches_points"][k], "receiver")
        ridx = point_dirs(rp, ctr, wall_of, scene["dirs_out"])
        dist = np.linalg.norm(ctr - rp, axis=1)
        pw = np.zeros((n, nb, nt))
        lib().orc_collect(n, nd, nb, nt, _p(e), _p(_c(ridx, np.int32)), _p(_c(rfac, float)), _p(_c(dist, float)),
                          ctypes.c_double(c), ctypes.c_double(dt), _p(_c(att, float)), _p(pw))
        out[r] = pw if patchwise else np.sum(pw, axis=0)
    return out


def solve(scene, src_pos, receivers, c, dt, duration, max_order):
    """Full pipeline: bake, init, exchange, collect (mono)."""
    bk = bake(scene)
    e0dir, d0, svis = init_source(scene, bk, np.asarray(src_pos, float))
    nt = int(duration / dt)
    etot = exchange(scene, bk, e0dir, d0, c, dt, nt, max_order)
    mono = collect(scene, bk, etot, receivers, c, dt)
    return dict(bake=bk, e0dir=e0dir, d0=d0, svis=svis, etot=etot, mono=mono)


# ------------------------------------------------- CPU-baseline timing samples
def visibility_rows_sample(ctr, normals, points, i0, i1, stride, full=False):
    """Rows i0, i0 + stride, ... < i1 of the visibility matrix (geometry.py:750-797 loop).

    Returns (visible count, rows (R, N) uint8).  ``full`` evaluates every
    j != i of a row (the symmetric matrix's row), else only j > i.
    """
    lib().orc_patch_visibility_rows.restype = ctypes.c_longlong
    ctr, normals, points = _c(ctr, float), _c(normals, float), _c(points, float)
    n = ctr.shape[0]
    rows = np.zeros((len(range(int(i0), int(i1), int(stride))), n), dtype=np.uint8)
    cnt = int(lib().orc_patch_visibility_rows(n, points.shape[1], _p(ctr), _p(normals), _p(points), int(i0), int(i1),
                                              int(stride), int(bool(full)), _p(rows)))
    return cnt, rows


def exchange_rows_out(nd, nb, nt, prev_rows, prev_row_of_pair, dst_off, delay, fprime, att_fac, slot, s_in, brdf,
                      rows):
    """One exchange order (RadiosityFast.py:1121-1143) for destination `rows`, written out (R, nd, nb, nt) FP64.

    prev_rows: float32 (M, nb, nt) source rows of the previous order;
    prev_row_of_pair[e] is the row pair e reads (its source patch and
    outgoing direction).  Pairs are destination-major (dst_off, (N + 1,)).
    """
    rows = _c(rows, np.int32)
    out = np.zeros((rows.size, nd, nb, nt))
    args = [_c(prev_rows, np.float32), _c(prev_row_of_pair, np.int64), _c(dst_off, np.int64), _c(delay, np.int32),
            _c(fprime, float), _c(att_fac, float), _c(slot, np.int32), _c(s_in, np.int32), _c(brdf, float)]
    lib().orc_exchange_rows_out(nd, nb, nt, _p(args[0]), _p(args[1]), _p(args[2]), _p(args[3]), _p(args[4]),
                                _p(args[5]), _p(args[6]), _p(args[7]), _p(args[8]), brdf.shape[1], rows.size,
                                _p(rows), _p(out))
    return out


def exchange_rows_sample(nd, nb, nt, prev, dst_off, src, p2o, delay, fprime, att_fac, slot, s_in, brdf, rows):
    """One exchange order for the given destination rows (RadiosityFast.py:1121-1143 loop)."""
    lib().orc_exchange_rows_sample.restype = ctypes.c_double
    args = [_c(prev, float), _c(dst_off, np.int64), _c(src, np.int32), _c(p2o, np.int32), _c(delay, np.int32),
            _c(fprime, float), _c(att_fac, float), _c(slot, np.int32), _c(s_in, np.int32), _c(brdf, float),
            _c(rows, np.int32)]
    prev_rows = args[0].shape[0]
    return float(lib().orc_exchange_rows_sample(nd, nb, nt, _p(args[0]), prev_rows, _p(args[1]), _p(args[2]),
                                                _p(args[3]), _p(args[4]), _p(args[5]), _p(args[6]), _p(args[7]),
                                                _p(args[8]), _p(args[9]), brdf.shape[1], len(rows), _p(args[10])))
