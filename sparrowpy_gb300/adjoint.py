"""Gradients of receiver energy-decay losses with respect to the materials.

Materials are the tables of create_from_scattering (sparrowpy/brdf.py:8-130)
stored x pi (RadiosityFast.py:815), one per BRDF slot, with per-slot,
per-band absorption a and scattering s:

    BRDF_slot[c, o, b] = (1 - a[slot, b]) (s[slot, b] + (1 - s[slot, b]) K_c [o == m_c])

(m_c: mirror direction of incoming direction c, K_c = pi / (cos w) as in
brdf.py:110-118).  `DifferentiableExchange` runs the forward solve (the
same CUDA path as DirectionalRadiosityFast, FP32 histograms, or FP64 when
the radiosity object's precision is "fp64") and, behind a
torch.autograd.Function, the hand-written adjoint of the exchange
(libsparrow_gb300: sp_adjoint_*) in the same precision.  The FP64 form
serves as the reference gradient of the FP32 one.  Exchange states are checkpointed every m
orders on the forward pass (the smallest m whose states fit in device
memory; sqrt(K) when memory is short) and recomputed segment by segment on
the backward pass.  The reference has no differentiable path.
"""
import ctypes
import itertools
import math

import numpy as np
import torch

from . import _native as nat
from .brdf import create_from_scattering
from .coords import Coordinates, FrequencyData, _cart
from .radiosity import _ptr, _stream, receiver_tile_order

_PLAN_TAGS = itertools.count(1)  # plan reuse tags: one per backward pass (process-wide, never 0)


def mirror_table(directions):
    """(mirror_of_in (n,), gain (n,)) of the create_from_scattering table x pi for one direction set.

    gain[c] = K_c, the specular table value per unit (1 - a)(1 - s); -1 / 0
    where an incoming direction has no mirror entry.
    """
    one = FrequencyData(np.zeros(1), np.array([1000.0]))
    tab = np.asarray(create_from_scattering(directions, directions, one, one).freq)[..., 0] * np.pi
    m = np.argmax(tab, axis=1)
    gain = tab[np.arange(tab.shape[0]), m]
    has = gain > 0
    return np.where(has, m, -1).astype(np.int32), np.where(has, gain, 0.0)


def material_tables(alpha, scattering, mirror, gain, n_out):
    """(S, n_in, n_out, B) float64 tables (1 - a)(s + (1 - s) K_c [o == m_c]) on alpha's device."""
    dev = alpha.device
    n_in = mirror.shape[0]
    spec = torch.zeros((n_in, n_out), dtype=torch.float64, device=dev)
    has = np.nonzero(mirror >= 0)[0]
    spec[torch.as_tensor(has, device=dev), torch.as_tensor(mirror[has], dtype=torch.long, device=dev)] = \
        torch.as_tensor(gain[has], dtype=torch.float64, device=dev)
    a = alpha.to(torch.float64)[:, None, None, :]
    s = scattering.to(torch.float64)[:, None, None, :]
    return (1.0 - a) * (s + (1.0 - s) * spec[None, :, :, None])


def energy_decay_loss(mono, target, eps=1e-30):
    """sum_{r, b, t} (log EDC_model - log EDC_target)^2, EDC = reverse cumulative sum over t."""
    edc = torch.flip(torch.cumsum(torch.flip(mono, [-1]), -1), [-1])
    edc_t = torch.flip(torch.cumsum(torch.flip(target, [-1]), -1), [-1])
    return torch.sum((torch.log(edc + eps) - torch.log(edc_t + eps)) ** 2)


class DifferentiableExchange:
    """Receiver histograms as a differentiable function of per-slot absorption and scattering.

    radiosity: a DirectionalRadiosityFast (precision "fp32" or "fp64") whose walls use
    one direction set `directions` (the unrotated Coordinates their tables
    were built from); bake_geometry is run here once.  slot_of_wall maps each
    wall to its material slot (default: wall index).  Calling the object
    with alpha, scattering (n_slots, n_bins) tensors returns the mono
    receiver histograms (R, B, T) float64 on the device.
    """

    def __init__(self, radiosity, directions, source, receivers, speed_of_sound, etc_time_resolution, etc_duration,
                 max_reflection_order, slot_of_wall=None, checkpoint_every=None):
        r = radiosity
        self.r = r
        self.prec = nat.SP_F64 if r.precision == "fp64" else nat.SP_F32
        self.dtype = torch.float64 if r.precision == "fp64" else torch.float32
        self.esz = 8 if r.precision == "fp64" else 4
        self.source = source
        self.receivers = np.atleast_2d(np.asarray(receivers, dtype=float).reshape(-1, 3))
        self.c = float(speed_of_sound)
        self.dt = float(etc_time_resolution)
        self.nt = int(etc_duration / etc_time_resolution)
        self.K = int(max_reflection_order)
        self._m_fixed = int(checkpoint_every) if checkpoint_every else None
        self.m = self._m_fixed or max(1, int(math.ceil(math.sqrt(self.K))))
        self.slot_of_wall = np.arange(r.n_walls) if slot_of_wall is None else np.asarray(slot_of_wall, dtype=int)
        self.n_slots = int(self.slot_of_wall.max()) + 1
        mirror, gain = mirror_table(directions)
        self.mirror_np, self.gain_np = mirror, gain
        self.n_out = _cart(directions).reshape(-1, 3).shape[0]
        dev = r.device
        self.mirror = torch.as_tensor(mirror, device=dev)
        self.gain = torch.as_tensor(gain, dtype=torch.float64, device=dev)
        if r._bake is None:
            r.bake_geometry()
        r.init_source_energy(source)  # e0 and d0 (the tables set on the walls only give E0dir's directions)
        self._c_src = self._source_incoming_index()
        self._slot_of_patch = torch.as_tensor(self.slot_of_wall[r._patch_to_wall_ids], dtype=torch.long,
                                              device=dev)
        self._slot_of_wall_dev = torch.as_tensor(self.slot_of_wall, dtype=torch.int32, device=dev)
        self._ckpt = None
        self._e0dir = None
        if self._m_fixed is None:
            self.m = self._choose_spacing()

    def _choose_spacing(self, margin=24 << 30):
        """Smallest checkpoint spacing whose states fit in the free device memory (at least sqrt(K) otherwise).

        Stored states are (K // m + 1) checkpoints plus m - 1 recomputed ones
        per segment; fewer recomputed orders for a smaller m.
        """
        r = self.r
        n, nd, nb = r._dev["e0dir"].shape
        h = n * nd * nb * self.nt * self.esz
        p = int(r._bake["n_dir"])
        fw = nat.size("sp_energy_exchange_workspace", self.prec, nat.SP_EXCHANGE_MATERIAL, n, nd, nb, self.nt, p,
                      self.n_slots, self.mirror_np.size, 1 + self.mirror_np.size)
        adj = nat.size("sp_adjoint_workspace", self.prec, n, nd, nb, self.nt, p, int(self.receivers.shape[0]))
        free, _ = torch.cuda.mem_get_info(r.device)
        avail = free + torch.cuda.memory_reserved(r.device) - torch.cuda.memory_allocated(r.device)
        for m in range(1, self.K + 1):
            need = (self.K // m + 1) * h + (m if m > 1 else 0) * h + fw + adj + 2 * h + margin
            if need <= avail:
                return m
        return max(1, int(math.ceil(math.sqrt(self.K))))

    # ------------------------------------------------------------- forward
    def _args(self, alpha64, scat64, etc):
        """sp_exchange_args of the material exchange (SP_EXCHANGE_MATERIAL) for these materials."""
        r = self.r
        a = r._exchange_args(self.c, self.dt, self.nt, self.K, "dense", etc)
        a.algorithm = nat.SP_EXCHANGE_MATERIAL
        a.energy_0_dir = self._e0dir.data_ptr()
        a.mat_alpha = alpha64.data_ptr()
        a.mat_scattering = scat64.data_ptr()
        a.mat_mirror = self.mirror.data_ptr()
        a.mat_gain = self.gain.data_ptr()
        if "receiver_order" not in r._dev:
            r._dev["receiver_order"] = r._t(receiver_tile_order(r.patches_center, r.patches_normal), torch.int32)
        a.receiver_order = r._dev["receiver_order"].data_ptr()
        a.pair_dst = r._bake["dst"].data_ptr()
        a.brdf_index = self._slot_of_wall_dev.data_ptr()  # material slot of each wall
        a.n_slots = self.n_slots
        return a

    def _workspace(self, a):
        n, nd, nb = self._e0dir.shape
        wsz = nat.size("sp_energy_exchange_workspace", self.prec, nat.SP_EXCHANGE_MATERIAL, n, nd, nb, self.nt,
                       a.n_dir_pairs, a.n_slots, a.n_in_dirs, 1 + a.n_in_dirs)
        return self.r._workspace(wsz), wsz

    def _source_dir(self, alpha64, scat64):
        """E0dir[i, o, b] = e0[i, b] BRDF_slot(i)[c_i, o, b] (RadiosityFast.py:988-1034) for these materials."""
        r = self.r
        e0 = r._dev["e0"]
        c_src = self._c_src
        slot = self._slot_of_patch
        m = self.mirror[c_src].long()
        k = self.gain[c_src]
        a = alpha64[slot]
        s = scat64[slot]
        n, nb = e0.shape
        spec = torch.zeros((n, self.n_out), dtype=torch.float64, device=r.device)
        has = torch.nonzero(m >= 0).reshape(-1)
        spec[has, m[has]] = k[has]
        return (e0[:, None, :] * (1.0 - a)[:, None, :]) * (s[:, None, :] + (1.0 - s)[:, None, :] * spec[:, :, None])

    def _solve(self, alpha, scattering, keep_states):
        r = self.r
        self._ckpt = None  # the previous pass's checkpoints go before new ones are allocated
        alpha64 = alpha.detach().to(torch.float64).contiguous()
        scat64 = scattering.detach().to(torch.float64).contiguous()
        self._e0dir = self._source_dir(alpha64, scat64).contiguous()
        n, nd, nb = self._e0dir.shape
        etc = torch.empty((n, nd, nb, self.nt), dtype=self.dtype, device=r.device)
        a = self._args(alpha64, scat64, etc)
        states = None
        if keep_states:
            n_ck = self.K // self.m + 1
            states = torch.empty((n_ck, n, nd, nb, self.nt), dtype=self.dtype, device=r.device)
            a.states_out = states.data_ptr()
            a.states_every = self.m
        ws, wsz = self._workspace(a)
        nat.call("sp_energy_exchange", ctypes.byref(a), _ptr(ws), wsz, _stream())
        r._dev["etc"] = etc
        r._etc_time_resolution, r._speed_of_sound = self.dt, self.c
        r._etc_duration = self.nt * self.dt
        self._ckpt = states
        return r._collect_device(self.receivers)

    def _resume(self, alpha64, scat64, state_in, k_from, k_to, states):
        """Orders k_from + 1 .. k_to from E_{k_from}; states[i] = E_{k_from + i} for i >= 1 (states[0] is not
        written: it would repeat state_in)."""
        dummy = torch.empty((1,), dtype=self.dtype, device=self.r.device)
        a = self._args(alpha64, scat64, dummy)
        a.max_order = int(k_to)
        a.state_in = state_in.data_ptr()
        a.state_order = int(k_from)
        a.states_out = states.data_ptr()
        a.states_every = 1
        a.skip_total = 1
        a.plan_tag = self._tag  # one plan for every segment of this backward pass
        ws, wsz = self._workspace(a)
        nat.call("sp_energy_exchange", ctypes.byref(a), _ptr(ws), wsz, _stream())

    def __call__(self, alpha, scattering):
        return _ExchangeFunction.apply(alpha, scattering, self)

    def forward_only(self, alpha, scattering):
        """Receiver histograms without keeping checkpoints (no gradient)."""
        with torch.no_grad():
            return self._solve(alpha, scattering, keep_states=False)

    # ------------------------------------------------------------ backward
    def _backward(self, alpha, scattering, grad_mono):
        r = self.r
        dev = r.device
        n, nd, nb = r._dev["e0dir"].shape
        nt, K, m = self.nt, self.K, self.m
        alpha64 = alpha.detach().to(torch.float64).contiguous()
        scat64 = scattering.detach().to(torch.float64).contiguous()
        self._tag = next(_PLAN_TAGS)
        ga = torch.zeros_like(alpha64)
        gs = torch.zeros_like(scat64)
        ridx, rfac, rdist = r._receiver_factors(self.receivers)
        gm = grad_mono.detach().to(torch.float64).contiguous()
        etc_dummy = torch.empty((1,), dtype=self.dtype, device=dev)
        fwd = self._args(alpha64, scat64, etc_dummy)
        state = nat.AdjointState()
        a = nat.AdjointArgs()
        a.fwd = ctypes.pointer(fwd)
        a.mirror_of_in = self.mirror.data_ptr()
        a.mirror_gain = self.gain.data_ptr()
        a.alpha = alpha64.data_ptr()
        a.scattering = scat64.data_ptr()
        a.n_receivers = int(self.receivers.shape[0])
        a.recv_dir = ridx.data_ptr()
        a.recv_factor = rfac.data_ptr()
        a.recv_dist = rdist.data_ptr()
        a.grad_mono = gm.data_ptr()
        a.grad_alpha = ga.data_ptr()
        a.grad_scattering = gs.data_ptr()
        a.state = ctypes.pointer(state)
        wsz = nat.size("sp_adjoint_workspace", self.prec, n, nd, nb, nt, fwd.n_dir_pairs,
                       int(self.receivers.shape[0]))
        ws = torch.empty((wsz,), dtype=torch.uint8, device=dev)
        st = _stream()
        nat.call("sp_adjoint_begin", ctypes.byref(a), _ptr(ws), wsz, st)
        seg_states = torch.empty((m, n, nd, nb, nt), dtype=self.dtype, device=dev) if m > 1 else None
        for seg in range((K - 1) // m, -1, -1):
            k_lo = seg * m                      # checkpointed state E_{k_lo}
            k_hi = min(k_lo + m, K)             # orders k_hi .. k_lo + 1 need E_{k_hi - 1} .. E_{k_lo}
            if k_hi - 1 > k_lo:
                self._resume(alpha64, scat64, self._ckpt[seg], k_lo, k_hi - 1, seg_states)
            for k in range(k_hi, k_lo, -1):
                e_prev = self._ckpt[seg] if k - 1 == k_lo else seg_states[k - 1 - k_lo]
                nat.call("sp_adjoint_order", ctypes.byref(a), _ptr(e_prev), _ptr(ws), wsz, st)
        g_e0 = torch.empty((n, nd, nb), dtype=torch.float64, device=dev)
        nat.call("sp_adjoint_finish", ctypes.byref(a), _ptr(g_e0), _ptr(ws), wsz, st)
        self._source_term(alpha64, scat64, g_e0, ga, gs)
        self._ckpt = None  # the checkpoints serve one backward pass
        return ga, gs

    def _source_term(self, alpha, scat, g_e0, ga, gs):
        """dL/d(a, s) through E0dir[i, o, b] = e0[i, b] BRDF_slot(i)[c_i, o, b] (RadiosityFast.py:988-1034)."""
        r = self.r
        dev = r.device
        e0 = r._dev["e0"]  # (N, B)
        c_src = self._c_src
        m_src = self.mirror[c_src].long()
        k_src = self.gain[c_src]
        slot = self._slot_of_patch
        g_sum = g_e0.sum(dim=1)  # (N, B)
        has = m_src >= 0
        g_m = torch.zeros_like(g_sum)
        idx = torch.nonzero(has).reshape(-1)
        g_m[idx] = g_e0[idx, m_src[idx], :]
        a_i, s_i = alpha[slot], scat[slot]
        k = (k_src * has)[:, None]
        ga.index_add_(0, slot, -e0 * (s_i * g_sum + (1.0 - s_i) * k * g_m))
        gs.index_add_(0, slot, e0 * (1.0 - a_i) * (g_sum - k * g_m))

    def _source_incoming_index(self):
        """Incoming-direction index of the source at each patch: argmin |d - unit(src - c)| over its wall's
        rotated directions, first index on ties (RadiosityFast.py:1359-1390)."""
        r = self.r
        bs = r._brdf_device()
        d = r._geometry()
        src = torch.as_tensor(np.asarray(self.source.cartesian, dtype=float).reshape(3), dtype=torch.float64,
                              device=r.device)
        v = src[None, :] - d["centers"]
        v = v / torch.linalg.norm(v, dim=1, keepdim=True)
        dirs = bs["dirs_in"][d["wall_of"].long()]  # (N, n_in, 3)
        dist = ((dirs - v[:, None, :]) ** 2).sum(-1)
        return torch.argmin(dist, dim=1)


class _ExchangeFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, alpha, scattering, solver):
        ctx.solver = solver
        ctx.save_for_backward(alpha, scattering)
        return solver._solve(alpha.detach(), scattering.detach(), keep_states=True)

    @staticmethod
    def backward(ctx, grad_mono):
        alpha, scattering = ctx.saved_tensors
        ga, gs = ctx.solver._backward(alpha, scattering, grad_mono)
        return ga.to(alpha.dtype), gs.to(scattering.dtype), None


def per_patch_room(dims, patch_size, directions, n_bins, precision="fp32"):
    """Shoebox with one wall per patch (per-patch materials), directions set on every wall."""
    from .geometry import shoebox_room_stub
    from .scenes import _patch_polygons
    from .radiosity import DirectionalRadiosityFast
    walls = _patch_polygons(shoebox_room_stub(*dims), patch_size)
    r = DirectionalRadiosityFast.from_polygon(walls, patch_size, precision=precision)
    freqs = np.arange(1, n_bins + 1) * 500.0
    one = FrequencyData(np.zeros(n_bins), freqs)
    table = create_from_scattering(directions, directions, FrequencyData(np.full(n_bins, 0.5), freqs), one)
    r.set_wall_brdf(np.arange(r.n_walls), table, directions, directions)
    r.set_air_attenuation(FrequencyData(np.zeros(n_bins), freqs))
    return r


def as_source(xyz):
    x = np.asarray(xyz, dtype=float).reshape(3)
    return Coordinates(x[0], x[1], x[2])
