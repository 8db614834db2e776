"""Universal form factors on the GPU (sparrowpy/form_factor/universal.py).

`patch2patch_ff_universal` takes the reference's arguments and returns its
(n_patches, n_patches) matrix with the visible pairs filled in (source i,
receiver j: the Stokes integral over i's area, or the Nusselt analogue for
pairs that share a vertex).  It runs sp_form_factors in FP64, the
reference's arithmetic; `universal_form_factor` is the same for one pair.
The point factors of a source and a receiver (`_source2patch_energy_universal`,
`_patch2receiver_energy_universal`, universal.py:98-160) run
sp_source_energy and sp_receiver_factors.  Patches are triangles to octagons
(all of one vertex count).
"""
import ctypes

import numpy as np
import torch

from .. import _native as nat
from ._dev import dev as _dev, ptr as _ptr, stream as _stream


def patch2patch_ff_universal(patches_points, patches_normals, patches_areas, visible_patches):
    """Form factors (n_patches, n_patches) of the listed (source, receiver) pairs (universal.py:12-52)."""
    pts = np.asarray(patches_points, dtype=float)
    n, nv = pts.shape[0], pts.shape[1]
    if pts.ndim != 3 or pts.shape[2] != 3 or not 3 <= nv <= 8:
        raise ValueError("patches_points must be (n_patches, 3..8, 3)")
    pairs = np.asarray(visible_patches, dtype=np.int32).reshape(-1, 2)
    out = np.zeros((n, n))
    m = pairs.shape[0]
    if m == 0:
        return out
    if pairs.min() < 0 or pairs.max() >= n:
        raise IndexError("visible_patches holds a patch index outside patches_points")
    p = _dev(pts, torch.float64)
    nr = _dev(np.asarray(patches_normals, dtype=float).reshape(n, 3), torch.float64)
    ar = _dev(np.asarray(patches_areas, dtype=float).reshape(n), torch.float64)
    pr = _dev(pairs, torch.int32)
    ff = torch.empty((m,), dtype=torch.float64, device="cuda")
    method = torch.empty((m,), dtype=torch.uint8, device="cuda")
    wsz = nat.size("sp_form_factors_workspace", n, m)
    ws = torch.empty((max(wsz, 1),), dtype=torch.uint8, device="cuda")
    nat.call("sp_form_factors", nat.SP_F64, n, nv, m, ctypes.c_void_p(pr.data_ptr()), ctypes.c_void_p(p.data_ptr()),
             ctypes.c_void_p(nr.data_ptr()), ctypes.c_void_p(ar.data_ptr()), ctypes.c_void_p(ff.data_ptr()),
             ctypes.c_void_p(method.data_ptr()), ctypes.c_void_p(ws.data_ptr()), wsz,
             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    out[pairs[:, 0], pairs[:, 1]] = ff.cpu().numpy()
    return out


def universal_form_factor(source_pts, source_normal, source_area, receiver_pts, receiver_normal):
    """Form factor from a source patch to a receiver patch (universal.py:54-96)."""
    pts = np.stack([np.asarray(source_pts, float), np.asarray(receiver_pts, float)])
    nrm = np.stack([np.asarray(source_normal, float), np.asarray(receiver_normal, float)])
    return float(patch2patch_ff_universal(pts, nrm, np.array([float(source_area), 0.0]), [[0, 1]])[0, 1])


def _source2patch_energy_universal(source_position, patches_center, patches_points, source_visibility,
                                   air_attenuation, n_bins):
    """(energy (n, n_bins), distance (n)) of each visible patch from a point source (universal.py:98-147):
    exp(-air_attenuation d) times the point factor; zeros for patches the source does not see."""
    pts = np.asarray(patches_points, dtype=float)
    n, nv = pts.shape[0], pts.shape[1]
    nb = int(n_bins)
    energy, distance = np.zeros((n, nb)), np.zeros(n)
    vis = np.asarray(source_visibility, dtype=bool).reshape(n)
    if n == 0 or not vis.any():
        return energy, distance
    att = np.zeros(nb) if air_attenuation is None else np.broadcast_to(
        np.asarray(air_attenuation, dtype=float).reshape(-1), (nb,))
    one = dict(wall=_dev(np.zeros(n), torch.int32), slot=_dev(np.zeros(1), torch.int32),
               dirs=_dev(np.array([[[0.0, 0.0, 1.0]]]), torch.float64), brdf=_dev(np.ones((1, 1, 1, nb)), torch.float64))
    e0 = torch.empty((n, nb), dtype=torch.float64, device="cuda")
    d0 = torch.empty((n,), dtype=torch.float64, device="cuda")
    e0dir = torch.empty((n, 1, nb), dtype=torch.float64, device="cuda")
    src, ctr, p = (_dev(np.asarray(source_position, float).reshape(3), torch.float64),
                   _dev(np.asarray(patches_center, float).reshape(n, 3), torch.float64), _dev(pts, torch.float64))
    v, a = _dev(vis.astype(np.uint8), torch.uint8), _dev(att, torch.float64)
    nat.call("sp_source_energy", _ptr(src), n, _ptr(ctr), _ptr(p), nv, _ptr(v), nb, _ptr(a), _ptr(one["wall"]),
             _ptr(one["slot"]), 1, _ptr(one["dirs"]), 1, _ptr(one["brdf"]), _ptr(e0), _ptr(d0), _ptr(e0dir), _stream())
    energy[vis] = e0.cpu().numpy()[vis]
    distance[vis] = d0.cpu().numpy()[vis]
    return energy, distance


def _patch2receiver_energy_universal(receiver_pos, patches_points, receiver_visibility):
    """Point factor (n) of each visible patch toward a receiver (universal.py:149-160); 0 where not visible."""
    pts = np.asarray(patches_points, dtype=float)
    n, nv = pts.shape[0], pts.shape[1]
    vis = np.asarray(receiver_visibility, dtype=bool).reshape(n)
    out = np.zeros(n)
    if n == 0 or not vis.any():
        return out
    ctr = pts.sum(axis=1) / nv
    rfac = torch.empty((n,), dtype=torch.float64, device="cuda")
    ridx = torch.empty((n,), dtype=torch.int32, device="cuda")
    dist = torch.empty((n,), dtype=torch.float64, device="cuda")
    rcv, c, p = (_dev(np.asarray(receiver_pos, float).reshape(3), torch.float64), _dev(ctr, torch.float64),
                 _dev(pts, torch.float64))
    v = _dev(vis.astype(np.uint8), torch.uint8)
    # every device array is held in a local until the results are read: a temporary freed before the launch
    # could hand its memory to the next allocation, whose copy would then overwrite it
    wall = _dev(np.zeros(n), torch.int32)
    dirs = _dev(np.array([[[0.0, 0.0, 1.0]]]), torch.float64)
    nat.call("sp_receiver_factors", _ptr(rcv), n, _ptr(c), _ptr(p), nv, _ptr(v), _ptr(wall), 1, _ptr(dirs),
             _ptr(rfac), _ptr(ridx), _ptr(dist), _stream())
    out[vis] = rfac.cpu().numpy()[vis]
    return out
