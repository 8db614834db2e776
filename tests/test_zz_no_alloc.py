"""Allocation-free patch visibility (sp_patch_visibility_static) against sp_patch_visibility.

Collected last (file name) so that it also runs after every other GPU test
has used the device.  Tolerance: exact (visibility is boolean).  The
allocation-free entry point runs the single-pass kernel, so besides the
small golden scenes it is compared on the 5939-patch street canyon, with
both entry points' times printed.
"""
import os

import numpy as np
import pytest

from conftest import load_golden, radiosity_from_golden


def test_static_visibility_rejects_too_many_patches():
    from sparrowpy_gb300 import _native as nat
    if not os.path.exists(nat.LIB_PATH):
        pytest.skip("library not built")
    # the size check comes before any device work (no GPU needed)
    assert nat.lib().sp_patch_visibility_static(16385, 4, None, None, None, None, None) == nat.SP_ERR_WORKSPACE
    assert nat.lib().sp_patch_visibility_static(-1, 4, None, None, None, None, None) == nat.SP_ERR_ARG


@pytest.mark.gpu
def test_static_visibility_matches_workspace_entry_point():
    import torch
    from sparrowpy_gb300 import _native as nat
    stream = torch.cuda.current_stream().cuda_stream
    for name in ("shoebox_126", "rot", "cube"):  # different sizes in a row reuse the one scratch array
        g = load_golden(name)
        r = radiosity_from_golden(g, "fp64")
        d = r._geometry()
        n, nv = r.n_patches, g["patches_points"].shape[1]
        ref = torch.empty((n, n), dtype=torch.uint8, device="cuda")
        wsz = nat.size("sp_patch_visibility_workspace", n)
        ws = torch.empty((wsz,), dtype=torch.uint8, device="cuda")
        nat.call("sp_patch_visibility", n, nv, d["centers"].data_ptr(), d["normals"].data_ptr(),
                 d["pts"].data_ptr(), ref.data_ptr(), ws.data_ptr(), wsz, stream)
        for _ in range(2):  # two calls in a row
            out = torch.full((n, n), 7, dtype=torch.uint8, device="cuda")
            nat.call("sp_patch_visibility_static", n, nv, d["centers"].data_ptr(), d["normals"].data_ptr(),
                     d["pts"].data_ptr(), out.data_ptr(), stream)
            torch.cuda.synchronize()
            assert torch.equal(out, ref)
        np.testing.assert_array_equal(ref.cpu().numpy(), g["V"])


@pytest.mark.gpu
def test_static_visibility_matches_on_the_street_canyon():
    import torch
    from sparrowpy_gb300 import _native as nat
    from sparrowpy_gb300 import scenes
    st = torch.cuda.current_stream()
    r = scenes.street_canyon(seed=3)
    d = r._geometry()
    n, nv = r.n_patches, r._patches_points.shape[1]
    args = (n, nv, d["centers"].data_ptr(), d["normals"].data_ptr(), d["pts"].data_ptr())
    ref = torch.empty((n, n), dtype=torch.uint8, device="cuda")
    out = torch.empty((n, n), dtype=torch.uint8, device="cuda")
    wsz = nat.size("sp_patch_visibility_workspace", n)
    ws = torch.empty((wsz,), dtype=torch.uint8, device="cuda")
    ms = {}
    for name, call in (("sp_patch_visibility", lambda: nat.call("sp_patch_visibility", *args, ref.data_ptr(),
                                                               ws.data_ptr(), wsz, st.cuda_stream)),
                       ("sp_patch_visibility_static", lambda: nat.call("sp_patch_visibility_static", *args,
                                                                      out.data_ptr(), st.cuda_stream))):
        call()  # first call (and the static array's address lookup) untimed
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        call()
        e1.record(st)
        e1.synchronize()
        ms[name] = e0.elapsed_time(e1)
    print(f"street canyon, {n} patches: " + ", ".join(f"{k} {v:.1f} ms" for k, v in ms.items()))
    assert torch.equal(out, ref)
