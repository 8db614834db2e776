"""GB300 DirectionalRadiosityFast: the reference API over the CUDA library.

Drop-in for sparrowpy/classes/RadiosityFast.py:15-968.  Method names,
arguments, attribute names, error types and messages follow the reference;
the numeric work of every step runs in libsparrow_gb300.so on one CUDA
device (device memory and the stream come from PyTorch):

=============================  ==============================================
reference step                 CUDA entry points
=============================  ==============================================
bake_geometry  :369-433        sp_patch_geometry, sp_patch_visibility,
                               sp_visible_pairs, sp_form_factors,
                               sp_count_directed/sp_directed_pairs,
                               sp_pair_setup
init_source_energy :436-522    sp_point_visibility, sp_source_energy
calculate_energy_exchange      sp_energy_exchange
  :524-568
collect_energy_receiver_*      sp_point_visibility, sp_receiver_factors,
  :570-752                     sp_collect_receiver
=============================  ==============================================

`form_factors_tilde` (N, N, D, B) is never needed by the solver; the
attribute is materialised on access (sp_form_factors_tilde).

Extra keyword (not in the reference): ``precision`` = "fp32" (default; FP32
exchange and Stokes form factors, FP64 for shared-vertex and near pairs and
for pairs whose FP32 error indicator is too large) or "fp64" (FP64
throughout).
"""
import ctypes

import numpy as np
import torch

from . import _native as nat
from . import geometry as geo
from .coords import Coordinates, FrequencyData, TimeData, _cart, is_coordinates

_PREC = {"fp32": nat.SP_F32, "fp64": nat.SP_F64}
STRUCTURED_MAX_SAMPLES = 65535  # time bins the structured exchange kernels address (16-bit base delays)


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _pair_dir_tables(bs):
    """The BRDF state's direction tables with identical ones merged: (table of each wall, dirs_in, dirs_out).

    Walls of the same orientation have the same rotated direction sets.  The
    pair set-up looks a table up for every directed pair; with the tables
    merged (exact comparison) it reads a few small, cache-resident ones
    instead of one per wall, with the same results.
    """
    if "pair_tables" not in bs:
        n_w = bs["dirs_in"].shape[0]
        both = torch.cat([bs["dirs_in"].reshape(n_w, -1), bs["dirs_out"].reshape(n_w, -1)], dim=1)
        uniq, inv = torch.unique(both, dim=0, return_inverse=True)
        k = bs["n_in"] * 3
        bs["pair_tables"] = (inv.to(torch.int32), uniq[:, :k].reshape(-1, bs["n_in"], 3).contiguous(),
                             uniq[:, k:].reshape(-1, bs["n_out"], 3).contiguous())
    return bs["pair_tables"]


_SIDE_STREAMS = {}
_PREP_POOL = None


def _prep_pool():
    """One host worker thread for BRDF preparation that runs beside the bake's blocking calls."""
    global _PREP_POOL
    if _PREP_POOL is None:
        import concurrent.futures as cf
        _PREP_POOL = cf.ThreadPoolExecutor(max_workers=1)
    return _PREP_POOL


_COPY_POOL = None


def _copy_pool():
    global _COPY_POOL
    if _COPY_POOL is None:
        import concurrent.futures as cf
        _COPY_POOL = cf.ThreadPoolExecutor(max_workers=4)
    return _COPY_POOL


def _stack_tables(arrays, out=None):
    """np.stack of equally shaped float64 tables, joined in C (np.concatenate along the first axis).

    A scene with one wall per patch has thousands of BRDF slots; np.stack's
    per-array Python work would dominate its copy.  out: an optional
    destination of the stacked shape (e.g. pinned host memory).
    """
    first = arrays[0]
    if first.ndim == 0 or any(a.shape != first.shape for a in arrays):
        raise ValueError("all BRDF tables must have the same shape")
    n = len(arrays)
    if out is None:
        out = np.empty((n,) + first.shape)
    flat = out.reshape((n * first.shape[0],) + first.shape[1:])
    if n < 256:
        np.concatenate(arrays, axis=0, out=flat)
        return out
    # large tables: four chunks in parallel (numpy releases the GIL while it copies)
    k = first.shape[0]
    bounds = [(q * n // 4, (q + 1) * n // 4) for q in range(4)]
    list(_copy_pool().map(lambda ab: np.concatenate(arrays[ab[0]:ab[1]], axis=0, out=flat[ab[0] * k:ab[1] * k]),
                          bounds))
    return out


def _object_array(values):
    """A per-wall list (e.g. of Coordinates, as RadiosityFast.to_dict writes an object array) as a 1-D object
    array; arrays and None pass through."""
    if values is None or isinstance(values, np.ndarray):
        return values
    out = np.empty(len(values), dtype=object)
    for k, v in enumerate(values):
        out[k] = v
    return out


def _side_stream(device):
    """One side stream per device for host-bound preparation that overlaps the bake kernels."""
    key = torch.device(device).index
    if key not in _SIDE_STREAMS:
        _SIDE_STREAMS[key] = torch.cuda.Stream(device=device)
    return _SIDE_STREAMS[key]


def brdf_rows_host(brdf, rel_tol=1e-12):
    """Host restatement of sp_brdf_structure (the per-row step of analyse_brdf).

    brdf: (n_slots, n_in, n_out, n_bins).  Returns (diff, spec, target,
    scale, irregular): per row (slot, incoming direction) the median over the
    outgoing directions (diff, per band), the one outgoing direction deviating
    from it by more than rel_tol * max|brdf| (target, -1 if none) with its
    excess (spec), per slot and band max |brdf| (scale), and whether any row
    has more than one deviating direction.
    """
    brdf = np.asarray(brdf, dtype=float)
    S, Din, Dout, B = brdf.shape
    big = np.max(np.abs(brdf)) if brdf.size else 0.0
    tol = rel_tol * max(big, 1e-300)
    if Dout == 1:
        diff = brdf[:, :, 0, :]
        spec = np.zeros_like(diff)
        target = -np.ones((S, Din), dtype=np.int64)
        irregular = False
    else:
        if Dout >= 3:
            diff = np.sort(brdf, axis=2)[:, :, Dout // 2, :]
        else:
            diff = brdf[:, :, 0, :]
        dev = brdf - diff[:, :, None, :]
        any_out = (np.abs(dev) > tol).any(axis=3)
        irregular = bool(np.any(any_out.sum(axis=2) > 1))
        has = any_out.any(axis=2)
        target = np.where(has, np.argmax(any_out, axis=2), -1)
        tsafe = np.where(has, target, 0)
        spec = np.take_along_axis(dev, tsafe[:, :, None, None], axis=2)[:, :, 0, :]
        spec = np.where(has[:, :, None], spec, 0.0)
    scale = np.max(np.abs(brdf), axis=(1, 2)) if brdf.size else np.zeros((S, B))
    return diff, spec, target, scale, irregular


_ROW_HASH = np.random.default_rng(0x5EED).integers(1, 2 ** 63, size=4096, dtype=np.uint64) | np.uint64(1)


def _unique_rows(key):
    """First index and inverse of the distinct rows of a float matrix, as np.unique(axis=0) gives them.

    Rows are hashed exactly (their bits times odd 64-bit multipliers, summed
    modulo 2^64, with -0.0 taken as 0.0), the hashes made unique, and every
    row checked against its group's first row; the groups are then ranked by
    the lexicographic order of those rows.  A hash collision or an over-long
    row falls back to np.unique(axis=0).
    """
    S, K = key.shape
    if S == 0 or K > _ROW_HASH.size or np.isnan(key).any():
        _, first, inverse = np.unique(key, axis=0, return_index=True, return_inverse=True)
        return first, inverse.reshape(-1)
    key = np.ascontiguousarray(key, dtype=np.float64)
    bits = (key + 0.0).view(np.uint64)
    h = bits @ _ROW_HASH[:K]  # integer product: exact, wraps modulo 2^64
    _, first_h, inv_h = np.unique(h, return_index=True, return_inverse=True)
    inv_h = inv_h.reshape(-1)
    if not np.array_equal(key, key[first_h[inv_h]]):
        _, first, inverse = np.unique(key, axis=0, return_index=True, return_inverse=True)
        return first, inverse.reshape(-1)
    order = np.lexsort(key[first_h].T[::-1])  # first column most significant
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    return first_h[order], rank[inv_h]


def _fold_unused(key, used):
    """Rows of slots no wall uses take the first used slot's row, so that they form no group of their own."""
    if used is None or not np.any(used) or np.all(used):
        return key
    key = key.copy()
    key[~used] = key[np.argmax(used)]
    return key


def group_brdf_rows(diff, spec, target, scale, used=None):
    """Group slots whose normalised rows agree: BRDF = scale[slot, b] * (diff + spec [o == m]).

    Returns slot_group (S,), slot_scale (S, B), n_groups, class_diff /
    class_spec (G * n_in, B), class_target (G * n_in,) (-1 = no mirror term).
    used: optional (S,) mask of the slots some wall uses; the others join
    the first used slot's group.
    """
    diff, spec, target = np.asarray(diff, float), np.asarray(spec, float), np.asarray(target)
    S, Din, B = diff.shape
    scale = np.asarray(scale, float)
    scale = np.where(scale > 0, scale, 1.0)
    nd = diff / scale[:, None, :]
    ns = spec / scale[:, None, :]
    key = np.concatenate([np.round(nd.reshape(S, -1), 12), np.round(ns.reshape(S, -1), 12),
                          target.reshape(S, -1).astype(float)], axis=1)
    first, inverse = _unique_rows(_fold_unused(key, used))
    G = first.size
    reps = first
    class_diff = nd[reps].reshape(G * Din, B)
    class_spec = ns[reps].reshape(G * Din, B)
    class_target = target[reps].reshape(G * Din)
    return dict(slot_group=inverse.astype(np.int32), slot_scale=scale.astype(float), n_groups=int(G),
                class_diff=np.ascontiguousarray(class_diff), class_spec=np.ascontiguousarray(class_spec),
                class_target=class_target.astype(np.int32))


def group_brdf_tables(brdf, used=None):
    """Group slots whose whole tables agree up to a per-slot, per-band scale: BRDF[slot] = scale[slot, b] T_g.

    brdf: (n_slots, n_in, n_out, n_bins), any values.  Returns slot_group
    (S,), slot_scale (S, B) (max |brdf| per slot and band), n_groups and
    class_table (G * n_in, n_out, B): the normalised table row of class
    c = g * n_in + s.  For tables without the diffuse-plus-mirror structure
    (the general exchange contracts these rows on the device).
    """
    brdf = np.asarray(brdf, dtype=float)
    S, Din, Dout, B = brdf.shape
    scale = np.max(np.abs(brdf), axis=(1, 2)) if brdf.size else np.zeros((S, B))
    scale = np.where(scale > 0, scale, 1.0)
    norm = brdf / scale[:, None, None, :]
    first, inverse = _unique_rows(_fold_unused(np.round(norm.reshape(S, -1), 12), used))
    G = first.size
    return dict(slot_group=inverse.astype(np.int32), slot_scale=scale, n_groups=int(G),
                class_table=np.ascontiguousarray(norm[first].reshape(G * Din, Dout, B)))


def analyse_brdf(brdf, rel_tol=1e-12):
    """Factor BRDF tables as scale[slot, b] * (diff[g, s, b] + spec[g, s, b] [o == m[g, s]]) on the host.

    brdf: (n_slots, n_in, n_out, n_bins).  Returns None when some row has
    more than one outgoing direction off the row's common value (the dense
    exchange is used then), else the dict of group_brdf_rows.  The solver
    runs the row step on the GPU (sp_brdf_structure); this host version is
    its reference.
    """
    diff, spec, target, scale, irregular = brdf_rows_host(brdf, rel_tol)
    if irregular:
        return None
    return group_brdf_rows(diff, spec, target, scale)


def receiver_tile_order(centers, normals, bits=10):
    """Receiver order for the tiled exchange: grouped by normal, then Morton order.

    Consecutive groups of 16 receivers in this order form one tile; compact
    tiles of coplanar patches see a source in nearly the same direction and
    delay, which is what lets the exchange kernel reuse a loaded source
    window across the tile.
    """
    centers = np.asarray(centers, dtype=float)
    if centers.shape[0] == 0:
        return np.zeros(0, dtype=np.int32)
    lo = centers.min(axis=0)
    span = np.maximum(centers.max(axis=0) - lo, 1e-12)
    q = np.clip(((centers - lo) / span * ((1 << bits) - 1)).astype(np.int64), 0, (1 << bits) - 1)
    code = np.zeros(centers.shape[0], dtype=np.int64)
    for bit in range(bits):
        for axis in range(3):
            code |= ((q[:, axis] >> bit) & 1) << (3 * bit + axis)
    _, nid = np.unique(np.round(np.asarray(normals, float), 6), axis=0, return_inverse=True)
    return np.lexsort((code, nid.reshape(-1))).astype(np.int32)


class DirectionalRadiosityFast:
    """Radiosity object for directional scattering coefficients (GB300)."""

    def __init__(self, walls_points, walls_normal, walls_up_vector, patches_points, n_patches, patch_to_wall_ids,
                 visibility_matrix=None, visible_patches=None, form_factors=None, form_factors_tilde=None,
                 frequencies=None, brdf=None, brdf_index=None, brdf_incoming_directions=None,
                 brdf_outgoing_directions=None, patch_2_brdf_outgoing_index=None, air_attenuation=None,
                 speed_of_sound=None, etc_time_resolution=None, etc_duration=None, distance_patches_to_source=None,
                 energy_init_source=None, energy_exchange_etc=None, *, precision="fp32", device=None):
        if precision not in _PREC:
            raise ValueError("precision must be 'fp32' or 'fp64'")
        self.precision = precision
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device()) \
            if torch.cuda.is_available() else torch.device("cuda")
        walls_points = np.atleast_3d(np.asarray(walls_points, dtype=float))
        self._walls_points = walls_points
        self._walls_normal = np.atleast_2d(np.asarray(walls_normal, dtype=float))
        self._walls_up_vector = np.atleast_2d(np.asarray(walls_up_vector, dtype=float))
        self._patches_points = np.atleast_3d(np.asarray(patches_points, dtype=float))
        self._n_patches = int(n_patches)
        self._patch_to_wall_ids = np.atleast_1d(np.array(patch_to_wall_ids, dtype=int))
        self._frequencies = None if frequencies is None else np.array(frequencies)
        self._brdf = None if brdf is None else [np.array(b) for b in brdf]
        self._brdf_index = None if brdf_index is None else np.array(brdf_index, dtype=np.int64)
        self._brdf_incoming_directions = _object_array(brdf_incoming_directions)
        self._brdf_outgoing_directions = _object_array(brdf_outgoing_directions)
        self._air_attenuation = None if air_attenuation is None else np.array(air_attenuation, dtype=float)
        self._speed_of_sound = None if speed_of_sound is None else float(speed_of_sound)
        self._etc_time_resolution = None if etc_time_resolution is None else float(etc_time_resolution)
        self._etc_duration = None if etc_duration is None else float(etc_duration)
        self._source = None
        # host copies of results (filled lazily from the device, or given)
        self._host = {}
        for key, val in (("visibility_matrix", visibility_matrix), ("visible_patches", visible_patches),
                         ("form_factors", form_factors), ("form_factors_tilde", form_factors_tilde),
                         ("patch_2_brdf_outgoing_index", patch_2_brdf_outgoing_index),
                         ("distance_patches_to_source", distance_patches_to_source),
                         ("energy_init_source", energy_init_source), ("energy_exchange_etc", energy_exchange_etc)):
            if val is not None:
                self._host[key] = np.array(val)
        self._dev = {}      # device tensors of the current geometry / results
        self._bake = None   # device state of the last bake
        self.host_bytes_uploaded = 0  # host -> device bytes copied by this object
        self._dirs_xyz = None         # rotated direction sets as arrays (set_wall_brdf)
        # E_total as the last partial sum S_K of S_k = E_0 + M(S_{k-1}) (the
        # tiled exchanges): no per-order E_total update
        self.partial_sums = True
        # order-by-order E_total (partial_sums False, or exchange states
        # saved), FP32: the late bins (the second half of the histogram) are
        # summed over the orders with Kahan compensation
        self.compensated_total = True
        # general BRDF tables, FP32, 32 <= directions <= 64: the receiver-side
        # contraction on the tensor cores (False: on the CUDA cores)
        self.tensor_cores = True
        self._max_order = None
        self.check()

    # ------------------------------------------------------------ validation
    def check(self):
        """Check the input data for consistency (RadiosityFast.py:211-337)."""
        n_walls = self._walls_points.shape[0]
        if self._walls_points.shape[2] != 3:
            raise ValueError("Walls need to be of shape (n_walls, n_points, 3)")
        if self._walls_up_vector.shape != (n_walls, 3):
            raise ValueError("Up vector of walls need to be of shape (n_walls, 3)")
        if self._walls_normal.shape != (n_walls, 3):
            raise ValueError("Normal of walls need to be of shape (n_walls, 3)")
        if (self._patches_points.shape[0] != self.n_patches) or (self._patches_points.shape[2] != 3):
            raise ValueError("Patches need to be of shape (n_patches, n_points, 3)")
        if self._patch_to_wall_ids.shape != (self.n_patches,):
            raise ValueError("patch_to_wall_ids need to be of shape (n_patches,)")
        ids = set(self._patch_to_wall_ids.tolist())
        if any(i not in range(n_walls) for i in ids) or any(i not in ids for i in range(n_walls)):
            raise ValueError("patch_to_wall_ids does contain other ids than range(n_walls)")
        n_bins = 1
        if self._frequencies is not None:
            if len(self._frequencies.shape) != 1:
                raise ValueError("Frequencies need to be of shape (n_bins,)")
            n_bins = self._frequencies.size
        ff = self._host.get("form_factors")
        if ff is not None and ff.shape != (self.n_patches, self.n_patches):
            raise ValueError("form_factors need to be of shape (n_patches, n_patches)")
        n_out = 1
        if self._brdf_index is not None and len(self._brdf_index) != n_walls:
            raise ValueError("brdf_index need to be of shape (n_walls,)")
        if self._brdf_incoming_directions is not None:
            if any(not is_coordinates(i) for i in self._brdf_incoming_directions):
                raise ValueError("brdf_incoming_directions need to be a list of type pf.Coordinates")
        if self._brdf_outgoing_directions is not None:
            if any(not is_coordinates(i) for i in self._brdf_outgoing_directions):
                raise ValueError("brdf_outgoing_directions need to be a list of type pf.Coordinates")
            n_out = self._brdf_outgoing_directions[0].csize
        fft = self._host.get("form_factors_tilde")
        if fft is not None and fft.shape != (self.n_patches, self.n_patches, n_out, n_bins):
            raise ValueError("form_factors_tilde need to be of shape "
                             "(n_patches, n_patches, n_outgoing_directions, n_bins)")
        if self._air_attenuation is not None:
            if len(self._air_attenuation.shape) != 1 or self._air_attenuation.shape[0] != n_bins:
                raise ValueError("Air attenuation need to be of shape (n_bins,)")
        if self._speed_of_sound is not None and self._speed_of_sound <= 0:
            raise ValueError("Speed of sound must be positive and non-zero")
        if self._etc_time_resolution is not None and self._etc_time_resolution <= 0:
            raise ValueError("Time resolution must be positive and non-zero")
        if self._etc_duration is not None and self._etc_duration <= 0:
            raise ValueError("Duration must be positive and non-zero")
        d0 = self._host.get("distance_patches_to_source")
        if d0 is not None and d0.shape != (self.n_patches,):
            raise ValueError("distance_patches_to_source need to be of shape (n_patches,)")
        e0 = self._host.get("energy_init_source")
        if e0 is not None and e0.shape != (self.n_patches, n_out, n_bins):
            raise ValueError("energy_init_source need to be of shape (n_patches, n_outgoing_directions, n_bins)")
        etc = self._host.get("energy_exchange_etc")
        if etc is not None:
            n_samples = int(self._etc_duration / self._etc_time_resolution)
            if etc.shape != (self.n_patches, n_out, n_bins, n_samples):
                raise ValueError("energy_exchange_etc need to be of shape "
                                 "(n_patches, n_outgoing_directions, n_bins, n_samples)")

    # -------------------------------------------------------------- creation
    @classmethod
    def from_polygon(cls, polygon_list, patch_size, *, precision="fp32", device=None):
        """Create the object from wall polygons (RadiosityFast.py:340-367)."""
        counts = sorted({p.pts.shape[0] for p in polygon_list})
        if len(counts) > 1:
            raise ValueError(f"walls of different vertex counts {counts}: the wall arrays hold one count (as the "
                             "reference's); split the walls into polygons of one count, e.g. the triangles of a "
                             "mesh's fine version")
        walls_points = np.array([p.pts for p in polygon_list])
        walls_normal = np.array([p.normal for p in polygon_list])
        walls_up_vector = np.array([p.up_vector for p in polygon_list])
        patches_points, _, n_patches, patch_to_wall_ids = geo.process_patches(walls_points, walls_normal, patch_size)
        return cls(walls_points, walls_normal, walls_up_vector, patches_points, n_patches, patch_to_wall_ids,
                   precision=precision, device=device)

    def clone(self):
        """A new object with copies of this object's host-side inputs (no device state)."""
        r = DirectionalRadiosityFast(self._walls_points, self._walls_normal, self._walls_up_vector,
                                     self._patches_points, self._n_patches, self._patch_to_wall_ids,
                                     frequencies=self._frequencies, air_attenuation=self._air_attenuation,
                                     precision=self.precision, device=self.device)
        if self._brdf is not None:
            r._brdf = [np.array(b) for b in self._brdf]
            r._brdf_index = self._brdf_index.copy()
            r._brdf_incoming_directions = self._brdf_incoming_directions.copy()
            r._brdf_outgoing_directions = self._brdf_outgoing_directions.copy()
            a = self._dirs_xyz
            if a is not None and self._dirs_belong(a):
                r._dirs_xyz = dict(a, of=(r._brdf_incoming_directions, r._brdf_outgoing_directions))
        return r

    # ---------------------------------------------------------- device state
    def _t(self, arr, dtype):
        t = torch.as_tensor(np.ascontiguousarray(arr), dtype=dtype)
        self.host_bytes_uploaded += t.numel() * t.element_size()
        return t.to(self.device, non_blocking=False)

    def _geometry(self):
        d = self._dev
        if "pts" not in d:
            n = self.n_patches
            d["pts"] = self._t(self._patches_points, torch.float64)
            d["normals"] = self._t(self.patches_normal, torch.float64)
            d["wall_of"] = self._t(self._patch_to_wall_ids, torch.int32)
            d["walls_pts"] = self._t(self._walls_points, torch.float64)
            d["walls_normal"] = self._t(self._walls_normal, torch.float64)
            d["centers"] = torch.empty((n, 3), dtype=torch.float64, device=self.device)
            d["areas"] = torch.empty((n,), dtype=torch.float64, device=self.device)
            nat.call("sp_patch_geometry", n, self._patches_points.shape[1], _ptr(d["pts"]), _ptr(d["centers"]),
                     _ptr(d["areas"]), _stream())
        return d

    def _brdf_key(self):
        return (id(self._brdf), len(self._brdf), tuple(self._brdf_index.tolist()))

    def _cached_brdf(self):
        """The device BRDF state if it still matches the object's tables, else None."""
        cached = self._dev.get("brdf_state")
        if cached is not None and cached["key"] == self._brdf_key():
            return cached
        return None

    def _brdf_device(self):
        """Device copies of the current BRDF tables and direction sets."""
        if self._brdf_incoming_directions is None:
            return None
        cached = self._cached_brdf()
        if cached is not None:
            return cached
        key = self._brdf_key()
        if np.any(self._brdf_index < 0):
            raise ValueError("every wall needs a BRDF (set_wall_brdf) before this step")
        din, dout = self._direction_arrays()
        slots = []
        for b in self._brdf:
            b = np.asarray(b, dtype=float)
            if b.ndim == 1:  # default BRDF: one value per band (RadiosityFast.py:459-467)
                b = b.reshape(1, 1, -1)
            slots.append(b)
        shape = (len(slots),) + slots[0].shape
        if int(np.prod(shape)) >= (1 << 20):
            # large tables (one per wall of a per-patch material): stacked straight into pinned host memory
            # (the caching host allocator keeps it for the next object) and copied without a staging pass
            pinned = torch.empty(shape, dtype=torch.float64, pin_memory=True)
            brdf = _stack_tables(slots, out=pinned.numpy())
            dev_brdf = pinned.to(self.device, non_blocking=True)
            self.host_bytes_uploaded += pinned.numel() * pinned.element_size()
            torch.cuda.current_stream(self.device).synchronize()  # brdf_host may outlive this call
        else:
            brdf = _stack_tables(slots)
            dev_brdf = self._t(brdf, torch.float64)
        state = dict(key=key, n_in=din.shape[1], n_out=dout.shape[1], n_slots=brdf.shape[0], brdf_host=brdf,
                     dirs_in=self._t(din, torch.float64), dirs_out=self._t(dout, torch.float64),
                     brdf=dev_brdf, brdf_index=self._t(self._brdf_index, torch.int32))
        self._dev["brdf_state"] = state
        return state

    def _prepare_brdf(self, consumer=None):
        """Device BRDF tables and their diffuse-plus-mirror structure, made on a side stream.

        Stacking, uploading and grouping new tables is host work; bake_geometry
        runs it in a worker thread while its own thread waits in the
        visibility and form-factor calls, since none of it reads the geometry.
        The consumer stream (the one that uses the tables; default: the
        calling thread's current stream, which a worker thread must be given)
        then waits for the side stream, and the tables are recorded as used
        on it.
        """
        if self._brdf_incoming_directions is None:
            return None
        cached = self._cached_brdf()
        if cached is not None and "structure" in cached:
            return cached
        main = consumer if consumer is not None else torch.cuda.current_stream(self.device)
        side = _side_stream(self.device)
        with torch.cuda.device(self.device), torch.cuda.stream(side):
            bs = self._brdf_device()
            self._brdf_structure(bs)
        main.wait_stream(side)
        for v in bs.values():
            if isinstance(v, torch.Tensor) and v.is_cuda:
                v.record_stream(main)
        return bs

    def _used_slots(self, n_slots):
        """(n_slots,) mask of the BRDF slots some wall refers to (tables replaced later stay in the list)."""
        used = np.zeros(n_slots, dtype=bool)
        if self._brdf_index is not None:
            idx = np.asarray(self._brdf_index)
            used[idx[(idx >= 0) & (idx < n_slots)]] = True
        return used

    def _brdf_structure(self, bs):
        """Diffuse-plus-mirror structure of the current BRDF tables (None if absent), kept with them.

        The row step runs on the device (sp_brdf_structure); grouping the
        slots works on the small per-row results on the host.
        """
        if "structure" in bs:
            return bs["structure"]
        S, Din, Dout = bs["n_slots"], bs["n_in"], bs["n_out"]
        B = bs["brdf"].shape[-1]
        dev = self.device
        diff = torch.empty((S, Din, B), dtype=torch.float64, device=dev)
        spec = torch.empty((S, Din, B), dtype=torch.float64, device=dev)
        target = torch.empty((S, Din), dtype=torch.int32, device=dev)
        scale = torch.empty((S, B), dtype=torch.float64, device=dev)
        n_irr = torch.empty((1,), dtype=torch.int32, device=dev)
        wsz = nat.size("sp_brdf_structure_workspace")
        ws = torch.empty((wsz,), dtype=torch.uint8, device=dev)
        nat.call("sp_brdf_structure", S, Din, Dout, B, _ptr(bs["brdf"]), 1e-12, _ptr(diff), _ptr(spec),
                 _ptr(target), _ptr(scale), _ptr(n_irr), _ptr(ws), wsz, _stream())
        if int(n_irr.item()) > 0:
            st = None
        else:
            st = group_brdf_rows(diff.cpu().numpy(), spec.cpu().numpy(), target.cpu().numpy(), scale.cpu().numpy(),
                                 used=self._used_slots(S))
        bs["structure"] = st
        return st

    # ------------------------------------------------------------------ bake
    def bake_geometry(self):
        """Bake the geometry by calculating all the form factors (RadiosityFast.py:369-433)."""
        if not 3 <= self._patches_points.shape[1] <= 8:
            raise NotImplementedError("the form factor kernels support patches of 3 to 8 vertices")
        d = self._geometry()
        n = self.n_patches
        nv = self._patches_points.shape[1]
        st = _stream()
        dev = self.device
        # visibility (geometry.py:750-797)
        vis = torch.empty((n, n), dtype=torch.uint8, device=dev)
        wsz = nat.size("sp_patch_visibility_workspace", n)
        ws = torch.empty((max(wsz, 1),), dtype=torch.uint8, device=dev)
        # the BRDF tables are stacked, uploaded and grouped in a host thread on
        # a side stream while this thread waits in the visibility and
        # form-factor calls (ctypes and numpy release the GIL there)
        brdf_job = _prep_pool().submit(self._prepare_brdf, torch.cuda.current_stream(dev))
        nat.call("sp_patch_visibility", n, nv, _ptr(d["centers"]), _ptr(d["normals"]), _ptr(d["pts"]), _ptr(vis),
                 _ptr(ws), wsz, st)
        # visible pair list (RadiosityFast.py:377-387)
        cap = max(n * (n - 1) // 2, 1)
        pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
        pair_index = torch.full((n, n), -1, dtype=torch.int32, device=dev)
        row_counts = torch.empty((max(n, 1),), dtype=torch.int32, device=dev)
        row_off = torch.empty((n + 1,), dtype=torch.int64, device=dev)
        nat.call("sp_visible_pairs", n, _ptr(vis), _ptr(row_counts), _ptr(row_off), _ptr(pairs), _ptr(pair_index), st)
        n_vis = int(row_off[n].item()) if n > 0 else 0
        pairs = pairs[:n_vis].contiguous()
        # form factors (universal.py:12-52)
        ff = torch.zeros((max(n_vis, 1),), dtype=torch.float64, device=dev)
        method = torch.zeros((max(n_vis, 1),), dtype=torch.uint8, device=dev)
        fsz = nat.size("sp_form_factors_workspace", n, n_vis)
        fws = torch.empty((max(fsz, 1),), dtype=torch.uint8, device=dev)
        nat.call("sp_form_factors", _PREC[self.precision], n, nv, n_vis, _ptr(pairs), _ptr(d["pts"]),
                 _ptr(d["normals"]), _ptr(d["areas"]), _ptr(ff), _ptr(method), _ptr(fws), fsz, st)
        del fws
        self._bake_pairs(vis, pairs, pair_index, n_vis, ff, method, brdf_job.result)
        for k in ("visibility_matrix", "visible_patches", "form_factors", "form_factors_tilde",
                  "patch_2_brdf_outgoing_index"):
            self._host.pop(k, None)

    def _bake_pairs(self, vis, pairs, pair_index, n_vis, ff, method, brdf_state):
        """The bake after visibility and form factors: directed pairs, their directions, distances and F'.

        brdf_state: a callable giving the device BRDF state (or None).
        """
        d = self._geometry()
        n = self.n_patches
        st = _stream()
        dev = self.device
        # directed pairs, destination-major (RadiosityFast.py:1124-1131)
        sym = torch.empty((n, n), dtype=torch.uint8, device=dev)
        dcounts = torch.empty((max(n, 1),), dtype=torch.int32, device=dev)
        dst_off = torch.empty((n + 1,), dtype=torch.int64, device=dev)
        nat.call("sp_count_directed", n, _ptr(vis), _ptr(sym), _ptr(dcounts), _ptr(dst_off), st)
        n_dir = int(dst_off[n].item()) if n > 0 else 0
        src = torch.empty((max(n_dir, 1),), dtype=torch.int32, device=dev)
        dst = torch.empty((max(n_dir, 1),), dtype=torch.int32, device=dev)
        nat.call("sp_directed_pairs", n, _ptr(sym), _ptr(dst_off), _ptr(src), _ptr(dst), st)
        del sym
        # per-pair directions, distances and F' (RadiosityFast.py:402-414, 1234-1272, 538-543)
        bs = brdf_state()
        out_dir = torch.zeros((max(n_dir, 1),), dtype=torch.int32, device=dev)
        in_dir = torch.zeros((max(n_dir, 1),), dtype=torch.int32, device=dev)
        dist = torch.empty((max(n_dir, 1),), dtype=torch.float64, device=dev)
        unit_len = torch.empty((max(n_dir, 1),), dtype=torch.float64, device=dev)
        fprime = torch.empty((max(n_dir, 1),), dtype=torch.float64, device=dev)
        if bs:
            tab_of_wall, din_u, dout_u = _pair_dir_tables(bs)
            tab_of_patch = tab_of_wall[d["wall_of"].long()].contiguous()
        nat.call("sp_pair_setup", n_dir, n, _ptr(src), _ptr(dst), _ptr(d["centers"]), _ptr(d["areas"]),
                 _ptr(pair_index), _ptr(ff), _ptr(tab_of_patch) if bs else _ptr(d["wall_of"]),
                 bs["n_in"] if bs else 0, _ptr(din_u) if bs else _ptr(None),
                 bs["n_out"] if bs else 0, _ptr(dout_u) if bs else _ptr(None),
                 _ptr(out_dir), _ptr(in_dir), _ptr(dist), _ptr(unit_len), _ptr(fprime), st)
        att = None if self._air_attenuation is None else self._t(self._air_attenuation, torch.float64)
        n_bins = 1 if self._frequencies is None else self.n_bins
        self._bake = dict(vis=vis, pairs=pairs, pair_index=pair_index, n_vis=n_vis, ff=ff, ff_method=method,
                          dst_off=dst_off, src=src, dst=dst, n_dir=n_dir, out_dir=out_dir, in_dir=in_dir, dist=dist,
                          unit_len=unit_len, fprime=fprime, brdf=bs, att=att, n_bins=n_bins,
                          n_out=bs["n_out"] if bs else 1)

    def _restore_bake(self):
        """Device bake state from a visibility matrix and form factors held on the host (from_dict / from_read).

        The reference restores those attributes and exchanges without baking
        again; here the visible pairs, directed pairs and pair set-up are
        rebuilt from them (the O(N^3) visibility and the form factors are
        not recomputed).  Returns False when the host does not hold both.
        """
        vis_h = self._host.get("visibility_matrix")
        ff_h = self._host.get("form_factors")
        n = self.n_patches
        if vis_h is None or ff_h is None or np.shape(vis_h) != (n, n) or np.shape(ff_h) != (n, n):
            return False
        dev = self.device
        st = _stream()
        vis = self._t(np.triu(np.asarray(vis_h, dtype=bool), 1).astype(np.uint8), torch.uint8)
        cap = max(n * (n - 1) // 2, 1)
        pairs = torch.empty((cap, 2), dtype=torch.int32, device=dev)
        pair_index = torch.full((n, n), -1, dtype=torch.int32, device=dev)
        row_counts = torch.empty((max(n, 1),), dtype=torch.int32, device=dev)
        row_off = torch.empty((n + 1,), dtype=torch.int64, device=dev)
        nat.call("sp_visible_pairs", n, _ptr(vis), _ptr(row_counts), _ptr(row_off), _ptr(pairs), _ptr(pair_index), st)
        n_vis = int(row_off[n].item()) if n > 0 else 0
        pairs = pairs[:n_vis].contiguous()
        ij = pairs.cpu().numpy()
        ff = self._t(np.asarray(ff_h, dtype=float)[ij[:, 0], ij[:, 1]] if n_vis else np.zeros(1), torch.float64)
        method = torch.zeros((max(n_vis, 1),), dtype=torch.uint8, device=dev)
        self._bake_pairs(vis, pairs, pair_index, n_vis, ff, method, self._brdf_device)
        return True

    # ---------------------------------------------------------------- source
    def init_source_energy(self, source):
        """Initialize the source energy (RadiosityFast.py:436-522)."""
        if is_coordinates(source):
            if tuple(source.cshape) != (1,):
                raise ValueError('just one source position is allowed.')
            source_position = np.asarray(source.cartesian, dtype=float).reshape(-1, 3)[0]
        elif hasattr(source, "position"):
            source_position = np.asarray(source.position, dtype=float).reshape(3)
        else:
            raise ValueError("source must be a Coordinates or a SoundSource")
        self._source = source
        if self._brdf_incoming_directions is None:
            frequencies = np.array([0]) if self._frequencies is None else self._frequencies
            self.set_wall_brdf(np.arange(self.n_walls), FrequencyData(np.ones_like(frequencies, dtype=float),
                                                                      frequencies),
                               Coordinates(0, 0, 1, weights=1), Coordinates(0, 0, 1, weights=1))
            self._frequencies = frequencies
        if self._air_attenuation is None:
            frequencies = np.array([0]) if self._frequencies is None else self._frequencies
            self.set_air_attenuation(FrequencyData(np.zeros_like(frequencies, dtype=float), frequencies))
            self._frequencies = frequencies
        d = self._geometry()
        bs = self._brdf_device()
        n, nb = self.n_patches, self.n_bins
        st = _stream()
        dev = self.device
        src = self._t(source_position, torch.float64)
        svis = self._point_visibility(src)
        att = self._t(self._air_attenuation, torch.float64)
        e0 = torch.empty((n, nb), dtype=torch.float64, device=dev)
        d0 = torch.empty((n,), dtype=torch.float64, device=dev)
        e0dir = torch.empty((n, bs["n_out"], nb), dtype=torch.float64, device=dev)
        nat.call("sp_source_energy", _ptr(src), n, _ptr(d["centers"]), _ptr(d["pts"]), self._patches_points.shape[1],
                 _ptr(svis), nb, _ptr(att),
                 _ptr(d["wall_of"]), _ptr(bs["brdf_index"]), bs["n_in"], _ptr(bs["dirs_in"]), bs["n_out"],
                 _ptr(bs["brdf"]), _ptr(e0), _ptr(d0), _ptr(e0dir), st)
        directivity = getattr(source, "directivity", None)
        if directivity is not None and hasattr(source, "get_directivity"):
            centers = self.patches_center
            fac = np.stack([np.real(source.get_directivity(centers, self._frequencies[b])) for b in range(nb)], axis=-1)
            e0dir *= self._t(fac, torch.float64)[:, None, :]
        self._dev["svis"] = svis
        self._dev["e0dir"] = e0dir
        self._dev["e0"] = e0
        self._dev["d0"] = d0
        for k in ("distance_patches_to_source", "energy_init_source"):
            self._host.pop(k, None)

    def _point_visibility(self, points_dev):
        """Patch visibility from one point (3,) -> (N,) or from several (P, 3) -> (P, N), walls as blockers."""
        d = self._geometry()
        n = self.n_patches
        pts = points_dev.reshape(-1, 3).contiguous()
        n_p = pts.shape[0]
        out = torch.empty((n_p, max(n, 1)), dtype=torch.uint8, device=self.device)
        nw = self.n_walls
        wsz = nat.size("sp_point_visibility_workspace", nw)
        ws = torch.empty((max(wsz, 1),), dtype=torch.uint8, device=self.device)
        nat.call("sp_points_visibility", n_p, _ptr(pts), n, _ptr(d["centers"]), nw, self._walls_points.shape[1],
                 _ptr(d["walls_pts"]), _ptr(d["walls_normal"]), _ptr(out), _ptr(ws), wsz, _stream())
        return out[0] if points_dev.dim() == 1 else out

    # -------------------------------------------------------------- exchange
    def _exchange_plan(self):
        if self._bake is None:
            self._restore_bake()
        bk = self._bake
        if bk is None:
            raise ValueError("bake_geometry() must run before calculate_energy_exchange()")
        if "plan" in bk:
            return bk["plan"]
        bs = bk["brdf"]
        n_bins = bk["n_bins"]
        if bs is None:
            brdf = np.ones((1, 1, 1, n_bins))
            plan = dict(brdf=self._t(brdf, torch.float64), brdf_index=self._t(np.zeros(self.n_walls), torch.int32),
                        n_slots=1, n_in=1, n_out=1, host=brdf)
        else:
            plan = dict(brdf=bs["brdf"], brdf_index=bs["brdf_index"], n_slots=bs["n_slots"], n_in=bs["n_in"],
                        n_out=bs["n_out"], host=bs["brdf_host"])
        st = analyse_brdf(plan["host"]) if bs is None else self._brdf_structure(bs)
        # diffuse-plus-mirror tables: per (group, incoming direction) class when
        # the classes fit, else slot-wise (diffuse class + mirror-direction class)
        mode = None
        if st is not None:
            mode = "structured" if st["n_groups"] * plan["n_in"] <= 256 else \
                "slotwise" if 1 + plan["n_out"] <= 256 else None
        general = None
        if mode is None:
            # any other tables: per (group of proportional tables, incoming
            # direction) class, contracted with the full table rows
            general = group_brdf_tables(plan["host"], used=self._used_slots(plan["n_slots"]))
            n_class = general["n_groups"] * plan["n_in"]
            # the contraction keeps a tile's table rows in shared memory (at most 200 KB) and a bin's
            # outgoing directions in registers (at most 64)
            if n_class <= 256 and plan["n_out"] <= 64 and n_class * plan["n_out"] * 8 <= 190 * 1024:
                mode = "general"
        if mode is not None:
            plan["mode"] = mode
            if "receiver_order" not in self._dev:
                self._dev["receiver_order"] = self._t(
                    receiver_tile_order(self.patches_center, self.patches_normal), torch.int32)
            plan["receiver_order"] = self._dev["receiver_order"]
            if mode == "general":
                plan["structured"] = dict(
                    slot_group=self._t(general["slot_group"], torch.int32),
                    slot_scale=self._t(general["slot_scale"], torch.float64), n_groups=general["n_groups"],
                    class_table=self._t(general["class_table"], torch.float64))
            else:
                plan["structured"] = dict(
                    slot_group=self._t(st["slot_group"], torch.int32),
                    slot_scale=self._t(st["slot_scale"], torch.float64),
                    n_groups=st["n_groups"], class_diff=self._t(st["class_diff"], torch.float64),
                    class_spec=self._t(st["class_spec"], torch.float64),
                    class_target=self._t(st["class_target"], torch.int32))
        bk["plan"] = plan
        return plan

    def calculate_energy_exchange(self, speed_of_sound, etc_time_resolution, etc_duration, max_reflection_order=-1,
                                  recalculate=False, *, algorithm="auto"):
        """Calculate the energy exchange between patches (RadiosityFast.py:524-568)."""
        n_samples = int(etc_duration / etc_time_resolution)
        if self._dev.get("etc") is None and self._host.get("energy_exchange_etc") is None or recalculate:
            if "e0dir" not in self._dev:
                if self._host.get("energy_init_source") is None:
                    raise ValueError("init_source_energy() must run before calculate_energy_exchange()")
                self._dev["e0dir"] = self._t(self._host["energy_init_source"], torch.float64)
                self._dev["d0"] = self._t(self._host["distance_patches_to_source"], torch.float64)
            self._run_exchange(float(speed_of_sound), float(etc_time_resolution), n_samples,
                               int(max_reflection_order), algorithm)
            self._host.pop("energy_exchange_etc", None)
            self._max_order = int(max_reflection_order)
        self._etc_time_resolution = float(etc_time_resolution)
        self._speed_of_sound = float(speed_of_sound)
        self._etc_duration = float(etc_duration)

    def _init_only_args(self, c, dt, n_samples, etc):
        """Arguments of an exchange of order < 1: E_total is the source energy at its delays
        (RadiosityFast.py:550-556, _energy_exchange_init_energy :1037-1070).  It reads no pair
        data, so it needs no bake_geometry(), as in the reference."""
        d = self._geometry()
        bs = self._brdf_device()
        e0dir, d0 = self._dev["e0dir"], self._dev["d0"]
        n, nd, nb = e0dir.shape
        a = nat.ExchangeArgs()
        a.precision = _PREC[self.precision]
        a.algorithm = nat.SP_EXCHANGE_DENSE
        a.n_patches, a.n_dirs, a.n_bins, a.n_samples, a.max_order = n, nd, nb, n_samples, 0
        a.energy_0_dir = e0dir.data_ptr()
        a.distance_0 = d0.data_ptr()
        a.n_dir_pairs = 0
        a.wall_of = d["wall_of"].data_ptr()
        a.brdf_index = bs["brdf_index"].data_ptr()
        a.n_slots, a.n_in_dirs = bs["n_slots"], bs["n_in"]
        a.brdf = bs["brdf"].data_ptr()
        a.speed_of_sound, a.time_resolution = c, dt
        a.etc_total = etc.data_ptr()
        return a

    def _exchange_args(self, c, dt, n_samples, max_order, algorithm, etc):
        plan = self._exchange_plan()  # restores the bake from host state where needed
        bk = self._bake
        d = self._geometry()
        e0dir, d0 = self._dev["e0dir"], self._dev["d0"]
        n, nd, nb = e0dir.shape
        if nd != plan["n_out"] or nb != bk["n_bins"]:
            raise ValueError("the BRDF directions/bands changed after bake_geometry(); bake again")
        # the structured kernels pack base delays in 16 bits; longer histograms take the dense kernel
        fits = n_samples <= STRUCTURED_MAX_SAMPLES
        if algorithm not in ("auto", "dense", "structured", "slotwise", "general"):
            raise ValueError("algorithm must be 'auto', 'dense', 'structured', 'slotwise' or 'general'")
        tiled = algorithm in ("structured", "slotwise", "general")
        use_struct = "structured" in plan and (tiled or (algorithm == "auto" and fits))
        if tiled and "structured" not in plan:
            raise ValueError("BRDF tables have more than 256 (table group, incoming direction) classes")
        if tiled and not fits:
            raise ValueError(f"the structured exchange holds at most {STRUCTURED_MAX_SAMPLES} time bins")
        mode = plan.get("mode")
        if algorithm in ("structured", "slotwise") and mode == "general":
            raise ValueError("BRDF tables are not of the diffuse-plus-mirror form: use 'general'")
        if algorithm == "structured" and mode == "slotwise":
            raise ValueError("more than 256 (material group, incoming direction) classes: use 'slotwise'")
        if use_struct and algorithm in ("slotwise", "general"):
            mode = algorithm
        a = nat.ExchangeArgs()
        a.precision = _PREC[self.precision]
        a.algorithm = {"slotwise": nat.SP_EXCHANGE_SLOTWISE, "general": nat.SP_EXCHANGE_GENERAL}.get(
            mode, nat.SP_EXCHANGE_STRUCTURED) if use_struct else nat.SP_EXCHANGE_DENSE
        a.n_patches, a.n_dirs, a.n_bins, a.n_samples, a.max_order = n, nd, nb, n_samples, max_order
        a.energy_0_dir = e0dir.data_ptr()
        a.distance_0 = d0.data_ptr()
        a.n_dir_pairs = bk["n_dir"]
        a.dst_offset = bk["dst_off"].data_ptr()
        a.pair_src = bk["src"].data_ptr()
        a.pair_out_dir = bk["out_dir"].data_ptr()
        a.pair_in_dir = bk["in_dir"].data_ptr()
        a.pair_distance = bk["dist"].data_ptr()
        a.pair_fprime = bk["fprime"].data_ptr()
        a.pair_unit_len = bk["unit_len"].data_ptr()
        a.air_attenuation = bk["att"].data_ptr() if bk["att"] is not None else None
        a.wall_of = d["wall_of"].data_ptr()
        a.brdf_index = plan["brdf_index"].data_ptr()
        a.n_slots, a.n_in_dirs = plan["n_slots"], plan["n_in"]
        a.brdf = plan["brdf"].data_ptr()
        a.speed_of_sound, a.time_resolution = c, dt
        a.etc_total = etc.data_ptr()
        a.plain_total = 0 if self.compensated_total else 1
        a.no_tensor_cores = 0 if self.tensor_cores else 1
        a.partial_sums = 1 if (self.partial_sums and use_struct) else 0
        if use_struct:
            s = plan["structured"]
            a.slot_group = s["slot_group"].data_ptr()
            a.slot_scale = s["slot_scale"].data_ptr()
            a.n_groups = s["n_groups"]
            if "class_table" in s:
                a.class_table = s["class_table"].data_ptr()
            else:
                a.class_diff = s["class_diff"].data_ptr()
                a.class_spec = s["class_spec"].data_ptr()
                a.class_target = s["class_target"].data_ptr()
            a.receiver_order = plan["receiver_order"].data_ptr()
            a.pair_dst = bk["dst"].data_ptr()
        return a

    def _run_exchange(self, c, dt, n_samples, max_order, algorithm="auto", states=None, states_every=0):
        """Exchange of all orders; optional `states` (n, N, D, B, T) receives E_0, E_m, E_2m, ... (m = states_every)."""
        e0dir = self._dev["e0dir"]
        n, nd, nb = e0dir.shape
        dtype = torch.float32 if self.precision == "fp32" else torch.float64
        etc = torch.empty((n, nd, nb, n_samples), dtype=dtype, device=self.device)
        if max_order < 1 and states is None:
            a = self._init_only_args(c, dt, n_samples, etc)
        else:
            a = self._exchange_args(c, dt, n_samples, max_order, algorithm, etc)
        if states is not None:
            if a.algorithm not in (nat.SP_EXCHANGE_STRUCTURED, nat.SP_EXCHANGE_SLOTWISE, nat.SP_EXCHANGE_GENERAL):
                raise ValueError("saving exchange states needs the structured exchange")
            a.states_out = states.data_ptr()
            a.states_every = int(states_every)
            a.partial_sums = 0  # the states are the per-order energies E_k
        stats = (ctypes.c_int64 * 4)()
        a.plan_stats = stats
        order_ms = ctypes.c_float(-1.0)
        a.order_ms = ctypes.pointer(order_ms)
        scatter_ms = ctypes.c_float(-1.0)
        a.scatter_ms = ctypes.pointer(scatter_ms)
        n_class = 1 + nd if a.algorithm == nat.SP_EXCHANGE_SLOTWISE else a.n_groups * a.n_in_dirs
        wsz = nat.size("sp_energy_exchange_workspace", a.precision, a.algorithm, n, nd, nb, n_samples,
                       a.n_dir_pairs, a.n_slots, a.n_in_dirs, n_class)
        ws = self._workspace(wsz)
        rc = nat.lib().sp_energy_exchange(ctypes.byref(a), _ptr(ws), wsz, _stream())
        if rc == nat.SP_ERR_RANGE:
            raise IndexError("a source delay exceeds the histogram length (index out of bounds)")
        if rc != nat.SP_OK:
            raise nat.NativeError("sp_energy_exchange", rc)
        self._dev["etc"] = etc
        names = {nat.SP_EXCHANGE_STRUCTURED: "structured", nat.SP_EXCHANGE_SLOTWISE: "slotwise",
                 nat.SP_EXCHANGE_GENERAL: "general"}
        self.exchange_stats = dict(algorithm=names.get(a.algorithm, "dense"),
                                   source_groups=int(stats[0]), segments=int(stats[1]), pairs=int(stats[2]),
                                   tiles=int(stats[3]), order_ms=float(order_ms.value), orders=int(max_order),
                                   scatter_ms=float(scatter_ms.value), partial_sums=bool(a.partial_sums))

    def energy_balance(self):
        """FP64 per-band energy check of the last exchange (no counterpart in the reference).

        Returns a dict of per-band arrays: ``histogram`` = sum of E_total
        over patches, directions and bins (accumulated in FP64 on the GPU,
        sp_energy_totals), ``budget`` = the same total predicted without
        time by the orders' energy recursion through ff_tilde, from the
        source energy (sp_energy_budget, FP64), and ``rel_dev`` =
        |histogram - budget| / budget.  The two agree up to rounding when
        no contribution is delayed past the histogram's last bin (a closed
        room whose histogram outlasts the orders); otherwise the deviation
        is the energy beyond the histogram, which the reference drops
        (RadiosityFast.py:1137-1143).  Also ``ms``, the check's GPU time.
        """
        etc = self._etc_device()
        if self._max_order is None or self._max_order < 0 or "e0dir" not in self._dev:
            raise ValueError("calculate_energy_exchange() with max_reflection_order >= 0 must run first")
        n, nd, nb, nt = etc.shape
        dev = self.device
        st = _stream()
        stream = torch.cuda.current_stream(dev)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        hist = torch.empty((nb,), dtype=torch.float64, device=dev)
        wsz = nat.size("sp_energy_totals_workspace", nb)
        ws = torch.empty((wsz,), dtype=torch.uint8, device=dev)
        prec = nat.SP_F32 if etc.dtype == torch.float32 else nat.SP_F64
        nat.call("sp_energy_totals", prec, n * nd, nb, nt, _ptr(etc), _ptr(hist), _ptr(ws), wsz, st)
        budget = torch.empty((nb,), dtype=torch.float64, device=dev)
        if self._max_order >= 1:
            a = self._exchange_args(self._speed_of_sound, self._etc_time_resolution, nt, self._max_order, "dense",
                                    etc)
        else:
            a = self._init_only_args(self._speed_of_sound, self._etc_time_resolution, nt, etc)
        bsz = nat.size("sp_energy_budget_workspace", n, nd, nb, a.n_dir_pairs)
        bws = torch.empty((max(bsz, 1),), dtype=torch.uint8, device=dev)
        nat.call("sp_energy_budget", ctypes.byref(a), _ptr(budget), _ptr(bws), bsz, st)
        ev1.record(stream)
        ev1.synchronize()
        h, b = hist.cpu().numpy(), budget.cpu().numpy()
        return dict(histogram=h, budget=b, rel_dev=np.abs(h - b) / np.where(b > 0, b, 1.0),
                    ms=float(ev0.elapsed_time(ev1)))

    def _workspace(self, nbytes):
        ws = self._dev.get("ws")
        if ws is None or ws.numel() < nbytes:
            self._dev.pop("ws", None)
            ws = torch.empty((max(nbytes, 1),), dtype=torch.uint8, device=self.device)
            self._dev["ws"] = ws
        return ws

    def _etc_device(self):
        etc = self._dev.get("etc")
        if etc is None:
            host = self._host.get("energy_exchange_etc")
            if host is None:
                raise ValueError("calculate_energy_exchange() must run first")
            dtype = torch.float32 if self.precision == "fp32" else torch.float64
            etc = self._t(host, dtype)
            self._dev["etc"] = etc
        return etc

    # ------------------------------------------------------------- receivers
    def collect_energy_receiver_mono(self, receivers, direct_sound=False):
        """Collect the energy at the receivers (RadiosityFast.py:570-602)."""
        if not isinstance(direct_sound, bool):
            raise ValueError("direct_sound must be of type boolean")
        etc = self._collect(receivers, patchwise=False)
        if direct_sound:
            ds, n_delay = self.calculate_direct_sound(receivers)
            i_r = np.arange(len(n_delay))
            etc.time[i_r, :, n_delay] += ds
        return etc

    def calculate_direct_sound(self, receivers):
        """Direct sound at the receivers (RadiosityFast.py:605-657)."""
        if not is_coordinates(receivers):
            raise ValueError("Receiver positions must be of type pf.Coordinates")
        if is_coordinates(self._source):
            src = np.asarray(self._source.cartesian, float).reshape(-1, 3)[0]
        else:
            src = np.asarray(self._source.position, float).reshape(3)
        rc = np.asarray(receivers.cartesian, float).reshape(-1, 3)
        r = np.sqrt(np.sum((rc - src) ** 2, axis=-1))
        direct = np.ones((rc.shape[0], self.n_bins), dtype=float)
        direct *= (1 / (4 * np.pi * r ** 2))[:, np.newaxis]
        if self._air_attenuation is not None:
            for i in range(self.n_bins):
                direct[:, i] *= np.exp(-self._air_attenuation[i] * r)
        if not is_coordinates(self._source) and getattr(self._source, "directivity", None) is not None:
            for i in range(self.n_bins):
                direct[:, i] *= np.real(self._source.get_directivity(np.squeeze(rc), self._frequencies[i]))
        n_delay = np.array(r / self.speed_of_sound / self._etc_time_resolution, dtype=int)
        return direct, n_delay

    def collect_energy_receiver_patchwise(self, receivers):
        """Per-patch energy at the receivers (RadiosityFast.py:660-684)."""
        return self._collect(receivers, patchwise=True)

    def _collect_energy_patches(self, receiver_pos, propagation_fx=False):
        """Patch histograms as the receivers see them (RadiosityFast.py:686-752): (R, N, B, T) FP64.

        With propagation_fx each patch's histogram is delayed and attenuated
        towards the receiver (the patchwise collection); without, it is the
        patch's histogram in the receiver's direction times the point factor.
        """
        rc = np.atleast_2d(np.asarray(receiver_pos, dtype=float).reshape(-1, 3))
        if propagation_fx:
            return self._collect_device(rc, patchwise=True).cpu().numpy()
        etc = self._etc_device()
        ridx, rfac, _ = self._receiver_factors(rc)
        rows = etc[torch.arange(etc.shape[0], device=etc.device)[None, :], ridx.long()]  # (R, N, B, T)
        return (rows.double() * rfac[:, :, None, None]).cpu().numpy()

    def _collect(self, receivers, patchwise):
        if not is_coordinates(receivers):
            raise ValueError("Receiver positions must be of type pf.Coordinates")
        if patchwise and receivers.cdim != 1:
            raise ValueError("Receiver positions must be of shape (n_receivers, 3)")
        rc = np.atleast_2d(np.asarray(receivers.cartesian, dtype=float).reshape(-1, 3))
        data = self._collect_device(rc, patchwise).cpu().numpy()
        times = np.arange(data.shape[-1]) * self._etc_time_resolution
        return TimeData(data, times)

    def _collect_device(self, rc, patchwise=False):
        """Receiver histograms on the device, FP64: (R, B, T), or (R, N, B, T) patchwise."""
        etc = self._etc_device()
        bs = self._brdf_device()
        n, nd, nb, nt = etc.shape
        if bs is None or bs["n_out"] != nd:
            raise ValueError("the outgoing BRDF directions do not match the energy histograms")
        n_r = rc.shape[0]
        dev = self.device
        st = _stream()
        prec = nat.SP_F32 if etc.dtype == torch.float32 else nat.SP_F64
        att = self._t(self._air_attenuation if self._air_attenuation is not None else np.zeros(nb), torch.float64)
        if patchwise:
            out = torch.empty((n_r, n, nb, nt), dtype=torch.float64, device=dev)
        else:
            out = torch.empty((n_r, nb, nt), dtype=torch.float64, device=dev)
        ridx_all, rfac_all, dist_all = self._receiver_factors(rc)
        wsz = nat.size("sp_collect_workspace", n, nb)
        ws = torch.empty((max(wsz, 1),), dtype=torch.uint8, device=dev)
        for r in range(n_r):
            ridx, rfac, dist = ridx_all[r], rfac_all[r], dist_all[r]
            nat.call("sp_collect_receiver", prec, n, nd, nb, nt, _ptr(etc), _ptr(ridx), _ptr(rfac), _ptr(dist),
                     float(self.speed_of_sound), float(self._etc_time_resolution), _ptr(att),
                     _ptr(out[r]) if patchwise else _ptr(None), _ptr(None) if patchwise else _ptr(out[r]),
                     _ptr(ws), wsz, st)
        return out

    def _receiver_factors(self, rc):
        """Per receiver (rows of rc, (R, 3)) and patch: outgoing index, point factor, distance (R, N) each."""
        d = self._geometry()
        bs = self._brdf_device()
        n = self.n_patches
        n_r = rc.shape[0]
        dev = self.device
        st = _stream()
        ridx = torch.empty((n_r, n), dtype=torch.int32, device=dev)
        rfac = torch.empty((n_r, n), dtype=torch.float64, device=dev)
        dist = torch.empty((n_r, n), dtype=torch.float64, device=dev)
        rdev = self._t(rc, torch.float64)
        rvis = self._point_visibility(rdev)  # every receiver in one launch
        for r in range(n_r):
            nat.call("sp_receiver_factors", _ptr(rdev[r]), n, _ptr(d["centers"]), _ptr(d["pts"]),
                     self._patches_points.shape[1], _ptr(rvis[r]),
                     _ptr(d["wall_of"]), bs["n_out"], _ptr(bs["dirs_out"]), _ptr(rfac[r]), _ptr(ridx[r]),
                     _ptr(dist[r]), st)
        return ridx, rfac, dist

    # ------------------------------------------------------------- materials
    def set_air_attenuation(self, air_attenuation):
        """Set air attenuation factor in Np/m (RadiosityFast.py:754-764)."""
        self._check_set_frequency(air_attenuation.frequencies)
        self._air_attenuation = np.atleast_1d(np.asarray(air_attenuation.freq, dtype=float).squeeze())

    def set_wall_brdf(self, wall_indexes, brdf, incoming_directions, outgoing_directions):
        """Set the wall BRDF (RadiosityFast.py:766-816); stored times pi."""
        assert (np.asarray(incoming_directions.z) >= 0).all(), "Sources must be in the positive half space"
        assert (np.asarray(outgoing_directions.z) >= 0).all(), "Receivers must be in the positive half space"
        self._check_set_frequency(brdf.frequencies)
        if self._brdf_incoming_directions is None:
            self._brdf_incoming_directions = np.empty((self.n_walls), dtype=object)
            self._brdf_outgoing_directions = np.empty((self.n_walls), dtype=object)
            self._brdf_index = np.full((self.n_walls), -1, dtype=np.int64)
            self._brdf = []
        for i in np.atleast_1d(wall_indexes):
            inc, out = geo.rotate_coords_to_normal(self.walls_normal[i], self.walls_up_vector[i],
                                                   incoming_directions, outgoing_directions)
            self._brdf_incoming_directions[i] = inc
            self._brdf_outgoing_directions[i] = out
            self._note_wall_dirs(int(i), inc, out)
        self._brdf.append(np.asarray(brdf.freq, dtype=float) * np.pi)
        self._brdf_index[np.atleast_1d(wall_indexes)] = len(self._brdf) - 1
        self._dev.pop("brdf_state", None)

    def _note_wall_dirs(self, i, inc, out):
        """Keep (n_walls, n, 3) arrays of the rotated direction sets beside the Coordinates objects.

        They belong to the object arrays they were made for (held and compared
        by identity), so an assignment of new direction sets leaves them
        unused.
        """
        cin, cout = _cart(inc).reshape(-1, 3), _cart(out).reshape(-1, 3)
        a = self._dirs_xyz
        mine = a is not None and self._dirs_belong(a)
        if not mine or a["in"].shape[1:] != cin.shape or a["out"].shape[1:] != cout.shape:
            if mine and a["set"].any():
                self._dirs_xyz = None  # direction sets of different sizes: stacked from the objects
                return
            nw = self.n_walls
            a = dict(of=(self._brdf_incoming_directions, self._brdf_outgoing_directions), set=np.zeros(nw, dtype=bool),
                     **{"in": np.zeros((nw,) + cin.shape), "out": np.zeros((nw,) + cout.shape)})
            self._dirs_xyz = a
        a["in"][i], a["out"][i], a["set"][i] = cin, cout, True

    def _dirs_belong(self, a):
        return a["of"][0] is self._brdf_incoming_directions and a["of"][1] is self._brdf_outgoing_directions

    def _direction_arrays(self):
        """(n_walls, n_in, 3) and (n_walls, n_out, 3) rotated direction sets."""
        a = self._dirs_xyz
        if a is not None and self._dirs_belong(a) and a["set"].all():
            return a["in"], a["out"]
        return (np.array([_cart(c).reshape(-1, 3) for c in self._brdf_incoming_directions]),
                np.array([_cart(c).reshape(-1, 3) for c in self._brdf_outgoing_directions]))

    def _check_set_frequency(self, frequencies):
        frequencies = np.atleast_1d(np.asarray(frequencies))
        if self._frequencies is None:
            self._frequencies = frequencies
        else:
            assert self._frequencies.size == frequencies.size, "Number of frequency bins do not match"
            assert (self._frequencies == frequencies).all(), "Frequencies do not match"

    # ------------------------------------------------------------ state I/O
    def write(self, filename, compress=True):
        """Write the object to a state file (RadiosityFast.py:828-830): a zip of npy and JSON members (far.py)."""
        from . import far
        far.write(filename, self._state_values(), compress=compress)

    @classmethod
    def from_read(cls, filename, **kwargs):
        """Read an object from a state file (RadiosityFast.py:832-839); kwargs: precision, device.

        A file that holds the visibility matrix and the form factors needs no
        bake_geometry() before the next exchange.
        """
        from . import far
        data = far.read(filename)
        data = {k: (None if isinstance(v, str) and v == 'None' else v) for k, v in data.items()}
        return cls(**data, **kwargs)

    def _state_values(self):
        """The to_dict entries with arrays kept as arrays."""
        return {
            'walls_points': self._walls_points, 'walls_normal': self._walls_normal,
            'walls_up_vector': self._walls_up_vector, 'patches_points': self._patches_points,
            'n_patches': self._n_patches, 'patch_to_wall_ids': self._patch_to_wall_ids,
            'visibility_matrix': self._visibility_matrix, 'visible_patches': self._visible_patches,
            'form_factors': self._form_factors, 'form_factors_tilde': self._form_factors_tilde,
            'frequencies': self._frequencies, 'brdf': self._brdf, 'brdf_index': self._brdf_index,
            'brdf_incoming_directions': self._brdf_incoming_directions,
            'brdf_outgoing_directions': self._brdf_outgoing_directions,
            'patch_2_brdf_outgoing_index': self._patch_2_brdf_outgoing_index,
            'air_attenuation': self._air_attenuation, 'speed_of_sound': self._speed_of_sound,
            'etc_time_resolution': self._etc_time_resolution, 'etc_duration': self._etc_duration,
            'distance_patches_to_source': self._distance_patches_to_source,
            'energy_init_source': self._energy_init_source, 'energy_exchange_etc': self._energy_exchange_etc,
        }

    def to_dict(self) -> dict:
        """Convert the object to a dictionary (RadiosityFast.py:841-873)."""
        out = self._state_values()
        for key, value in out.items():
            if value is None:
                out[key] = 'None'
            elif isinstance(value, np.ndarray) and value.dtype != object:
                out[key] = value.tolist()
        return out

    @classmethod
    def from_dict(cls, input_dict: dict, **kwargs):
        """Create an object from a dictionary (RadiosityFast.py:882-886)."""
        d = {k: (None if isinstance(v, str) and v == 'None' else v) for k, v in input_dict.items()}
        return cls(**d, **kwargs)

    def __eq__(self, other):
        if not isinstance(other, DirectionalRadiosityFast):
            return False
        a, b = self.to_dict(), other.to_dict()
        if a.keys() != b.keys():
            return False
        for k in a:
            va, vb = a[k], b[k]
            if isinstance(va, (list, tuple, np.ndarray)) or isinstance(vb, (list, tuple, np.ndarray)):
                try:
                    if not np.array_equal(np.asarray(va, dtype=object if k.startswith('brdf_') else None),
                                          np.asarray(vb, dtype=object if k.startswith('brdf_') else None)):
                        return False
                except ValueError:
                    return False
            elif va != vb:
                return False
        return True

    # ------------------------------------------------- reference attributes
    def _host_get(self, key, make):
        if key not in self._host:
            val = make()
            if val is None:
                return None
            self._host[key] = val
        return self._host[key]

    @property
    def _visibility_matrix(self):
        return self._host_get("visibility_matrix",
                              lambda: None if self._bake is None else self._bake["vis"].cpu().numpy().astype(bool))

    @property
    def _visible_patches(self):
        return self._host_get("visible_patches",
                              lambda: None if self._bake is None else self._bake["pairs"].cpu().numpy().astype(np.int32))

    @property
    def _form_factors(self):
        def make():
            if self._bake is None:
                return None
            n = self.n_patches
            out = torch.empty((n, n), dtype=torch.float64, device=self.device)
            nat.call("sp_dense_form_factors", self._bake["n_vis"], n, _ptr(self._bake["pairs"]),
                     _ptr(self._bake["ff"]), _ptr(out), _stream())
            return out.cpu().numpy()
        return self._host_get("form_factors", make)

    @property
    def _form_factors_tilde(self):
        def make():
            bk = self._bake
            if bk is None:
                return None
            n = self.n_patches
            bs = bk["brdf"]
            nd = bk["n_out"]
            nb = bk["n_bins"]
            out = torch.empty((n, n, nd, nb), dtype=torch.float64, device=self.device)
            d = self._geometry()
            nat.call("sp_form_factors_tilde", bk["n_dir"], n, nd, nb, bs["n_in"] if bs else 1, _ptr(bk["src"]),
                     _ptr(bk["dst"]), _ptr(bk["in_dir"]), _ptr(bk["fprime"]), _ptr(bk["unit_len"]), _ptr(bk["att"]),
                     _ptr(d["wall_of"]), _ptr(bs["brdf_index"]) if bs else _ptr(None),
                     _ptr(bs["brdf"]) if bs else _ptr(None), _ptr(out), _stream())
            return out.cpu().numpy()
        return self._host_get("form_factors_tilde", make)

    @property
    def _patch_2_brdf_outgoing_index(self):
        def make():
            bk = self._bake
            if bk is None:
                return None
            n = self.n_patches
            if bk["brdf"] is None:
                return np.zeros((n, n), dtype=np.int64)
            out = torch.empty((n, n), dtype=torch.int64, device=self.device)
            nat.call("sp_outgoing_index_map", bk["n_dir"], n, _ptr(bk["src"]), _ptr(bk["dst"]), _ptr(bk["out_dir"]),
                     int(bk["n_out"]), _ptr(out), _stream())
            return out.cpu().numpy()
        return self._host_get("patch_2_brdf_outgoing_index", make)

    @property
    def _energy_init_source(self):
        return self._host_get("energy_init_source",
                              lambda: self._dev["e0dir"].cpu().numpy() if "e0dir" in self._dev else None)

    @property
    def _distance_patches_to_source(self):
        return self._host_get("distance_patches_to_source",
                              lambda: self._dev["d0"].cpu().numpy() if "d0" in self._dev else None)

    @property
    def _source_visibility(self):
        return self._dev["svis"].cpu().numpy().astype(bool) if "svis" in self._dev else None

    @property
    def _energy_exchange_etc(self):
        return self._host_get("energy_exchange_etc",
                              lambda: self._dev["etc"].cpu().numpy().astype(np.float64) if "etc" in self._dev else None)

    # ------------------------------------------------------------ properties
    @property
    def n_bins(self):
        return None if self._frequencies is None else self._frequencies.shape[0]

    @property
    def n_walls(self):
        return self._walls_points.shape[0]

    @property
    def n_patches(self):
        return self._n_patches

    @property
    def form_factors(self):
        return self._form_factors

    @property
    def visibility_matrix(self):
        return self._visibility_matrix

    @property
    def walls_area(self):
        return geo.calculate_area(self._walls_points)

    @property
    def walls_points(self):
        return self._walls_points

    @property
    def walls_normal(self):
        return self._walls_normal

    @property
    def walls_center(self):
        return geo.calculate_center(self._walls_points)

    @property
    def walls_up_vector(self):
        return self._walls_up_vector

    @property
    def patches_area(self):
        return geo.calculate_area(self._patches_points)

    @property
    def patches_center(self):
        return geo.calculate_center(self._patches_points)

    @property
    def patches_size(self):
        return geo.calculate_size(self._patches_points)

    @property
    def patches_points(self):
        return self._patches_points

    @property
    def patches_normal(self):
        return self._walls_normal[self._patch_to_wall_ids]

    @property
    def speed_of_sound(self):
        return self._speed_of_sound
