"""The C-ABI library loads and exports every symbol include/sparrow_gb300.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "sparrow_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b(sp_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("sp_patch_visibility", "sp_form_factors", "sp_energy_exchange", "sp_collect_receiver",
                 "sp_source_energy", "sp_pair_setup", "sp_visible_pairs"):
        assert must in names


def test_library_exports_all_declared_symbols():
    from sparrowpy_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        pytest.skip("library not built")
    lib = ctypes.CDLL(_native.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from sparrowpy_gb300 import _native
    assert set(declared_symbols()) == set(_native.exported_symbols())


def test_version_string():
    from sparrowpy_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        pytest.skip("library not built")
    assert b"sm_103a" in _native.lib().sp_version()


def test_workspace_queries_without_gpu():
    """Size queries are pure host arithmetic."""
    from sparrowpy_gb300 import _native as nat
    if not os.path.exists(nat.LIB_PATH):
        pytest.skip("library not built")
    a = nat.size("sp_energy_exchange_workspace", nat.SP_F32, nat.SP_EXCHANGE_DENSE, 10, 4, 2, 100, 50, 1, 4, 0)
    b = nat.size("sp_energy_exchange_workspace", nat.SP_F64, nat.SP_EXCHANGE_DENSE, 10, 4, 2, 100, 50, 1, 4, 0)
    assert b > a > 2 * 10 * 4 * 2 * 100 * 4
    s = nat.size("sp_energy_exchange_workspace", nat.SP_F32, nat.SP_EXCHANGE_STRUCTURED, 10, 4, 2, 100, 50, 1, 4, 4)
    assert s > 3 * 10 * 4 * 2 * 100 * 4
    assert nat.size("sp_patch_visibility_workspace", 100) >= 100 * 24


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    from sparrowpy_gb300 import _native
    monkeypatch.setattr(_native, "_lib", None)
    monkeypatch.setattr(_native, "LIB_PATH", str(tmp_path / "nope.so"))
    with pytest.raises(ImportError):
        _native.lib()


def test_struct_mirrors_match_the_library():
    """The ctypes mirrors have the C structs' sizes (a missing trailing field would be read as garbage)."""
    import ctypes as ct
    from sparrowpy_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        pytest.skip("library not built")
    lib = _native.lib()
    assert lib.sp_exchange_args_size() == ct.sizeof(_native.ExchangeArgs)
    assert lib.sp_adjoint_args_size() == ct.sizeof(_native.AdjointArgs)
    assert lib.sp_batch_args_size() == ct.sizeof(_native.BatchArgs)


def declared_prototypes():
    """name -> number of parameters, from the header's prototypes."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(sp_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_binding_argument_counts_match_header():
    """Every ctypes signature has as many arguments as its C prototype."""
    from sparrowpy_gb300 import _native
    protos = declared_prototypes()
    bad = {name: (len(args), protos[name]) for name, (_, args) in _native._SIGS.items()
           if name in protos and len(args) != protos[name]}
    assert not bad, bad
    assert len(protos) >= 30


def test_argument_checks_before_any_device_work():
    """Calls whose arguments the library refuses return SP_ERR_ARG before any CUDA call (so they run here):
    polygons of 2 or 9 vertices; partial sums together with saved per-order states."""
    import ctypes
    from sparrowpy_gb300 import _native as nat
    if not os.path.exists(nat.LIB_PATH):
        pytest.skip("library not built")
    lib = nat.lib()
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: the checks come first
    for nv in (2, 9):
        assert lib.sp_form_factors(nat.SP_F64, 4, nv, 1, fake, fake, fake, fake, fake, None, None, 0,
                                   None) == nat.SP_ERR_ARG
        assert lib.sp_source_energy(fake, 1, fake, fake, nv, fake, 1, fake, fake, fake, 1, fake, 1, fake, fake,
                                    fake, fake, None) == nat.SP_ERR_ARG
        assert lib.sp_receiver_factors(fake, 1, fake, fake, nv, fake, fake, 1, fake, fake, fake, fake,
                                       None) == nat.SP_ERR_ARG
    a = nat.ExchangeArgs()
    a.precision, a.algorithm = nat.SP_F32, nat.SP_EXCHANGE_STRUCTURED
    a.n_patches, a.n_dirs, a.n_bins, a.n_samples, a.max_order = 4, 2, 1, 100, 3
    a.n_dir_pairs, a.n_slots, a.n_in_dirs, a.n_groups = 4, 1, 2, 1
    a.speed_of_sound, a.time_resolution = 343.0, 1e-3
    for name in ("energy_0_dir", "distance_0", "etc_total", "wall_of", "brdf_index", "brdf", "dst_offset",
                 "pair_src", "pair_out_dir", "pair_in_dir", "pair_distance", "pair_fprime", "pair_unit_len",
                 "pair_dst", "slot_group", "slot_scale", "class_diff", "class_spec", "class_target"):
        setattr(a, name, 0x1000)
    a.states_out, a.states_every, a.partial_sums = 0x1000, 1, 1
    huge = 1 << 40  # the workspace check passes; nothing is touched before the argument checks
    assert lib.sp_energy_exchange(ctypes.byref(a), fake, huge, None) == nat.SP_ERR_ARG
