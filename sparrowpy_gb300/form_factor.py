"""Form factors between patches on the GPU (sparrowpy/form_factor/universal.py:12-96).

`patch2patch_ff_universal` takes the reference's arguments and returns its
(n_patches, n_patches) matrix with the visible pairs filled in (source i,
receiver j: the Stokes integral over i's area, or the Nusselt analogue for
pairs that share a vertex).  It runs sp_form_factors in FP64, the
reference's arithmetic; `universal_form_factor` is the same for one pair.
Patches are triangles to octagons (all of one vertex count).

The Kang closed forms of form_factor/kang.py (patch2patch_ff_kang and its
point factors) are not provided: DirectionalRadiosityFast does not use them,
and the Kang solver (kang.py) runs the forms of RadiosityKang.py.
"""
import ctypes

import numpy as np
import torch

from . import _native as nat


def _dev(a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


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
