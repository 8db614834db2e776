"""ctypes binding of libsparrow_gb300.so (the C ABI in include/sparrow_gb300.h).

The library must exist: there is no CPU fallback.  If it is missing the
import raises with the command that builds it.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsparrow_gb300.so")

SP_OK = 0
SP_ERR_ARG = -1
SP_ERR_CUDA = -2
SP_ERR_WORKSPACE = -3
SP_ERR_RANGE = -4
SP_ERR_TIMEOUT = -5
SP_ERR_UNSUPPORTED = -6
SP_F32 = 0
SP_F64 = 1
SP_EXCHANGE_DENSE = 0
SP_EXCHANGE_STRUCTURED = 1
SP_EXCHANGE_MATERIAL = 2
SP_EXCHANGE_SLOTWISE = 3
SP_EXCHANGE_GENERAL = 4

_ERRORS = {
    SP_ERR_ARG: "invalid argument",
    SP_ERR_CUDA: "CUDA launch or copy failed",
    SP_ERR_WORKSPACE: "workspace too small",
    SP_ERR_RANGE: "delay outside the histogram",
    SP_ERR_TIMEOUT: "bounded device wait gave up",
    SP_ERR_UNSUPPORTED: "unsupported configuration",
}

P = ctypes.c_void_p
I = ctypes.c_int
LL = ctypes.c_longlong
D = ctypes.c_double
SZ = ctypes.c_size_t


class ExchangeArgs(ctypes.Structure):
    """Mirror of `sp_exchange_args`."""
    _fields_ = [
        ("precision", I), ("algorithm", I),
        ("n_patches", I), ("n_dirs", I), ("n_bins", I), ("n_samples", I), ("max_order", I),
        ("energy_0_dir", P), ("distance_0", P),
        ("n_dir_pairs", LL),
        ("dst_offset", P), ("pair_src", P), ("pair_out_dir", P), ("pair_in_dir", P),
        ("pair_distance", P), ("pair_fprime", P), ("pair_unit_len", P),
        ("air_attenuation", P), ("wall_of", P), ("brdf_index", P),
        ("n_slots", I), ("n_in_dirs", I), ("brdf", P),
        ("speed_of_sound", D), ("time_resolution", D),
        ("etc_total", P),
        ("slot_group", P), ("slot_scale", P), ("n_groups", I),
        ("class_diff", P), ("class_spec", P), ("class_target", P),
        ("receiver_order", P), ("pair_dst", P), ("plan_stats", ctypes.POINTER(ctypes.c_int64)),
        ("order_ms", ctypes.POINTER(ctypes.c_float)),
        ("state_in", P), ("state_order", I), ("states_out", P), ("states_every", I), ("skip_total", I),
        ("mat_alpha", P), ("mat_scattering", P), ("mat_mirror", P), ("mat_gain", P),
        ("plan_tag", LL), ("scatter_ms", ctypes.POINTER(ctypes.c_float)), ("plain_total", I),
        ("class_table", P), ("no_tensor_cores", I), ("prepare_only", I), ("partial_sums", I),
    ]


class AdjointState(ctypes.Structure):
    """Mirror of `sp_adjoint_state` (host memory)."""
    _fields_ = [("ready", I), ("cur", I), ("n_active", ctypes.c_uint), ("n_groups", LL)]


class AdjointArgs(ctypes.Structure):
    """Mirror of `sp_adjoint_args`."""
    _fields_ = [
        ("fwd", ctypes.POINTER(ExchangeArgs)), ("mirror_of_in", P), ("mirror_gain", P),
        ("alpha", P), ("scattering", P), ("n_receivers", I), ("recv_dir", P), ("recv_factor", P),
        ("recv_dist", P), ("grad_mono", P), ("grad_alpha", P), ("grad_scattering", P),
        ("state", ctypes.POINTER(AdjointState)),
    ]


class BatchRoom(ctypes.Structure):
    """Mirror of `sp_batch_room` (host memory)."""
    _fields_ = [("args", ctypes.POINTER(ExchangeArgs)), ("ws", P), ("ws_bytes", SZ)]


class BatchArgs(ctypes.Structure):
    """Mirror of `sp_batch_args` (host memory)."""
    _fields_ = [("n_rooms", I), ("rooms", ctypes.POINTER(BatchRoom)), ("window_bins", I), ("ctas_per_sm", I),
                ("wait_limit", ctypes.c_uint), ("force_timeout", I), ("exchange_ms", ctypes.POINTER(ctypes.c_float)),
                ("items", ctypes.POINTER(ctypes.c_longlong)), ("wait_polls", ctypes.POINTER(ctypes.c_longlong))]


# name: (restype, argtypes)
_SIGS = {
    "sp_version": (ctypes.c_char_p, []),
    "sp_kernel_launches": (LL, []),
    "sp_exchange_args_size": (SZ, []),
    "sp_adjoint_args_size": (SZ, []),
    "sp_batch_args_size": (SZ, []),
    "sp_exchange_batch_workspace": (SZ, [I]),
    "sp_exchange_batch": (I, [ctypes.POINTER(BatchArgs), P, SZ, P]),
    "sp_patch_geometry": (I, [I, I, P, P, P, P]),
    "sp_patch_visibility_workspace": (SZ, [I]),
    "sp_patch_visibility": (I, [I, I, P, P, P, P, P, SZ, P]),
    "sp_patch_visibility_static": (I, [I, I, P, P, P, P, P]),
    "sp_point_visibility_workspace": (SZ, [I]),
    "sp_point_visibility": (I, [P, I, P, I, I, P, P, P, P, SZ, P]),
    "sp_points_visibility": (I, [I, P, I, P, I, I, P, P, P, P, SZ, P]),
    "sp_visible_pairs": (I, [I, P, P, P, P, P, P]),
    "sp_count_directed": (I, [I, P, P, P, P, P]),
    "sp_directed_pairs": (I, [I, P, P, P, P, P]),
    "sp_pair_setup": (I, [LL, I, P, P, P, P, P, P, P, I, P, I, P, P, P, P, P, P, P]),
    "sp_outgoing_index_map": (I, [LL, I, P, P, P, ctypes.c_int64, P, P]),
    "sp_form_factors_workspace": (SZ, [I, LL]),
    "sp_form_factors": (I, [I, I, I, LL, P, P, P, P, P, P, P, SZ, P]),
    "sp_dense_form_factors": (I, [LL, I, P, P, P, P]),
    "sp_form_factors_tilde": (I, [LL, I, I, I, I, P, P, P, P, P, P, P, P, P, P, P]),
    "sp_source_energy": (I, [P, I, P, P, I, P, I, P, P, P, I, P, I, P, P, P, P, P]),
    "sp_receiver_factors": (I, [P, I, P, P, I, P, P, I, P, P, P, P, P]),
    "sp_energy_exchange_workspace": (SZ, [I, I, I, I, I, I, LL, I, I, I]),
    "sp_energy_exchange": (I, [ctypes.POINTER(ExchangeArgs), P, SZ, P]),
    "sp_energy_totals_workspace": (SZ, [I]),
    "sp_energy_totals": (I, [I, LL, I, I, P, P, P, SZ, P]),
    "sp_energy_budget_workspace": (SZ, [I, I, I, LL]),
    "sp_energy_budget": (I, [ctypes.POINTER(ExchangeArgs), P, P, SZ, P]),
    "sp_adjoint_workspace": (SZ, [I, I, I, I, I, LL, I]),
    "sp_adjoint_begin": (I, [ctypes.POINTER(AdjointArgs), P, SZ, P]),
    "sp_adjoint_order": (I, [ctypes.POINTER(AdjointArgs), P, P, SZ, P]),
    "sp_adjoint_finish": (I, [ctypes.POINTER(AdjointArgs), P, P, SZ, P]),
    "sp_brdf_structure_workspace": (SZ, []),
    "sp_brdf_structure": (I, [I, I, I, I, P, D, P, P, P, P, P, P, SZ, P]),
    "sp_collect_workspace": (SZ, [I, I]),
    "sp_collect_receiver": (I, [I, I, I, I, I, P, P, P, P, D, D, P, P, P, P, SZ, P]),
    "sp_kang_init_energy": (I, [I, P, P, P, P, D, I, P, P, D, D, I, I, P, P, P]),
    "sp_kang_form_factors": (I, [I, P, P, P, I, P, P, P, D, P, P]),
    "sp_kang_exchange_workspace": (SZ, [I, I, I]),
    "sp_kang_exchange": (I, [I, I, I, I, I, P, P, P, P, P, I, P, P, P, LL, LL, D, D, P, SZ, P, P]),
    "sp_kang_receiver": (I, [I, P, P, I, I, I, P, I, P, P, D, D, P, P, P]),
    "sp_kang_directional_init_energy": (I, [I, P, P, P, P, D, I, P, P, D, D, I, I, I, P, P, P, P, P]),
    "sp_kang_directional_exchange": (I, [I, I, I, I, I, P, P, P, P, P, I, P, P, P, LL, LL, D, D, I, P, P, P, SZ, P,
                                         P]),
    "sp_kang_directional_receiver": (I, [I, P, P, I, I, I, P, I, P, P, D, D, I, P, P, P, P]),
    "sp_kang_pair_form_factors": (I, [LL, P, I, P, P, P, I, P, P]),
    "sp_kang_point_source": (I, [I, P, P, P, P, I, P, P, P, P, P]),
    "sp_kang_point_receiver": (I, [I, P, P, P, P]),
}


class NativeError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, name, code):
        super().__init__(f"{name} failed: {_ERRORS.get(code, 'unknown error')} (status {code})")
        self.code = code


_lib = None


def lib():
    """Load (once) and return the ctypes library handle."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` or "
                "`python sparrowpy_gb300/build_lib.py` (there is no CPU fallback)")
        h = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


def exported_symbols():
    return list(_SIGS)


def call(name, *args):
    """Call an int-returning entry point and raise NativeError on failure."""
    rc = getattr(lib(), name)(*args)
    if rc != SP_OK:
        raise NativeError(name, rc)
    return rc


def size(name, *args):
    return int(getattr(lib(), name)(*args))
