"""Kang form factors and point factors on the GPU (sparrowpy/form_factor/kang.py).

The closed forms for axis-aligned rectangular patches (Kang's method):
* `patch2patch_ff_kang` (kang.py:12-169): form factors of the listed
  (source, receiver) pairs, orthogonal pairs by Eq. 11-15, parallel pairs
  by Eq. 16, on sp_kang_pair_form_factors;
* `_source2patch_energy_kang` (kang.py:171-262): the energy a point source
  gives each patch, on sp_kang_point_source;
* `_patch2receiver_energy_kang` (kang.py:264-277): the receiver factor of
  each patch (Eq. 20), on sp_kang_point_receiver.
FP64 with the reference's operation order (unfused).
"""
import numpy as np
import torch

from .. import _native as nat
from ._dev import dev, ptr, stream


def patch2patch_ff_kang(patches_center, patches_normal, patches_size, visible_patches):
    """Form factors (n_patches, n_patches) of the listed (source, receiver) pairs; other entries 0."""
    ctr = np.asarray(patches_center, dtype=float).reshape(-1, 3)
    nrm = np.asarray(patches_normal, dtype=float).reshape(-1, 3)
    size = np.asarray(patches_size, dtype=float)
    n = ctr.shape[0]
    if size.ndim != 2 or size.shape[0] != n or size.shape[1] not in (2, 3):
        raise ValueError("patches_size must be (n_patches, 2) or (n_patches, 3)")
    pairs = np.asarray(visible_patches, dtype=np.int32).reshape(-1, 2)
    out = np.zeros((n, n))
    if pairs.shape[0] == 0:
        return out
    if pairs.min() < 0 or pairs.max() >= n:
        raise IndexError("visible_patches holds a patch index outside the patches")
    src, rcv = nrm[pairs[:, 0]], nrm[pairs[:, 1]]
    ortho = np.sum(rcv * src, axis=1) == 0
    if not np.all(np.any(np.abs(src[ortho]) > 1e-5, axis=1)) or not np.all(np.any(np.abs(rcv) > 1e-5, axis=1)):
        raise ValueError("a patch normal is zero")
    if size.shape[1] == 2 and np.any(ortho & (np.abs(src[:, 2]) <= 1e-5)):
        raise IndexError("orthogonal pairs read the third size column (as the reference's patches_size[i, 2])")
    ff = torch.empty((pairs.shape[0],), dtype=torch.float64, device="cuda")
    d_pairs, d_ctr, d_nrm, d_size = dev(pairs, torch.int32), dev(ctr), dev(nrm), dev(size)
    nat.call("sp_kang_pair_form_factors", pairs.shape[0], ptr(d_pairs), n, ptr(d_ctr), ptr(d_nrm), ptr(d_size),
             size.shape[1], ptr(ff), stream())
    out[pairs[:, 0], pairs[:, 1]] = ff.cpu().numpy()
    return out


def _source2patch_energy_kang(source_position, patches_center, patches_normal, air_attenuation, patches_size,
                              n_bins):
    """(energy (n, n_bins), distance (n)) of each axis-aligned patch from a point source."""
    ctr = np.asarray(patches_center, dtype=float).reshape(-1, 3)
    n, nb = ctr.shape[0], int(n_bins)
    energy, distance = np.empty((n, nb)), np.empty(n)
    if n == 0:
        return energy, distance
    e = torch.empty((n, nb), dtype=torch.float64, device="cuda")
    d = torch.empty((n,), dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    att = None if air_attenuation is None else dev(np.broadcast_to(
        np.asarray(air_attenuation, dtype=float).reshape(-1), (nb,)))
    d_src = dev(np.asarray(source_position, dtype=float).reshape(3))
    d_ctr = dev(ctr)
    d_nrm = dev(np.asarray(patches_normal, dtype=float).reshape(n, 3))
    d_size = dev(np.asarray(patches_size, dtype=float).reshape(n, 3))
    nat.call("sp_kang_point_source", n, ptr(d_src), ptr(d_ctr), ptr(d_nrm), ptr(d_size), nb, ptr(att), ptr(e),
             ptr(d), ptr(err), stream())
    if int(err.item()) == 3:
        raise ValueError("a patch normal is not along a coordinate axis")
    energy[:], distance[:] = e.cpu().numpy(), d.cpu().numpy()
    return energy, distance


def _patch2receiver_energy_kang(patch_receiver_distance, patches_normal):
    """Receiver factor (n) of each patch for its patch-to-receiver vector (n, 3)."""
    vec = np.asarray(patch_receiver_distance, dtype=float).reshape(-1, 3)
    n = vec.shape[0]
    if n == 0:
        return np.empty(0)
    f = torch.empty((n,), dtype=torch.float64, device="cuda")
    d_vec = dev(vec)
    d_nrm = dev(np.asarray(patches_normal, dtype=float).reshape(n, 3))
    nat.call("sp_kang_point_receiver", n, ptr(d_vec), ptr(d_nrm), ptr(f), stream())
    return f.cpu().numpy()
