"""Golden vectors for the Kang radiosity solver (sparrowpy/classes/RadiosityKang.py).

Two sources, both written to tests/golden/kang.npz:
* the reference's own stored results (tests/test_data/*.far of sparrowpy:
  form factors of parallel and perpendicular unit-cube walls, initial and
  exchanged energy matrices, the 10 x 20 x 15 m simulation at orders 2 and
  3), read from their npy members;
* a run of the reference's RadiosityKang here, on a 3 x 2 x 2 m room with
  0.5 m patches, two bands, air attenuation and per-wall scattering, with
  the stub modules of make_golden.py standing in for pyfar, sofar,
  deepdiff and matplotlib (not installed).  The per-wall energy matrices,
  form factors and the receiver response are stored raw (FP64).

Usage:  python tests/golden/make_kang_golden.py [--ref /path/to/sparrowpy]
"""
import argparse
import io
import json
import os
import sys
import zipfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from make_golden import import_reference  # noqa: E402

ROOM = dict(dims=(3.0, 2.0, 2.0), patch_size=0.5, max_order_k=4, ir_length_s=0.2, sampling_rate=1000,
            speed_of_sound=343.0, absorption=[0.1, 0.3], scattering=[[1.0, 0.9], [1.0, 1.0], [0.8, 1.0],
                                                                   [1.0, 1.0], [1.0, 0.7], [1.0, 1.0]],
            attenuation=[0.001, 0.004], source=[0.7, 0.6, 0.8], receiver=[2.2, 1.3, 1.1])


def far_arrays(path):
    """The npy members of a .far file (a zip), keyed by member name."""
    out = {}
    with zipfile.ZipFile(path) as z:
        for name in z.namelist():
            data = z.read(name)
            if data[:6] == b"\x93NUMPY":
                out[name] = np.load(io.BytesIO(data), allow_pickle=False)
    return out


def stored_results(test_data):
    out = {}
    for size in ("0.5", "1"):
        out[f"ff_parallel_size{size}"] = far_arrays(
            os.path.join(test_data, f"reference_form_factor_parallel_size{size}.far"))["form_factor/$ndarray"]
        out[f"E_init_size{size}"] = far_arrays(
            os.path.join(test_data, f"reference_matrix_directional_patch_size{size}.far"))["E_matrix/$ndarray"]
        out[f"E_exchange_size{size}"] = far_arrays(
            os.path.join(test_data, f"reference_energy_exchange_size{size}.far"))["E_matrix/$ndarray"]
    walls = [(i, j) for i in range(6) for j in range(6) if i // 2 != j // 2]
    for i, j in walls:
        out[f"ff_perpendicular_{i}_{j}_size0.5"] = far_arrays(
            os.path.join(test_data, f"reference_form_factor_perpendicular_{i}_{j}_size0.5.far"))["form_factor/$ndarray"]
    out["ff_perpendicular_0_0_size1"] = far_arrays(
        os.path.join(test_data, "reference_form_factor_perpendicular_0_0_size1.far"))["form_factor/$ndarray"]
    out["ff_perpendicular_sorted_size0.5"] = far_arrays(
        os.path.join(test_data, "reference_form_factor_perpendicular_size0.5.far"))["form_factor/$ndarray"]
    for k in (2, 3):
        a = far_arrays(os.path.join(test_data, f"simulation_X10_k{k}_5m.far"))
        out[f"sim_X10_k{k}_time"] = a["signal/_data"]
        out[f"sim_X10_k{k}_times"] = a["signal/_times"]
    return out


def reference_room(ref_path):
    import_reference(ref_path)
    import importlib
    kang = importlib.import_module("sparrowpy.classes.RadiosityKang")
    geo = importlib.import_module("sparrowpy.geometry")
    so = importlib.import_module("sparrowpy.sound_object")
    from sparrowpy_gb300.geometry import shoebox_room_stub
    walls = [geo.Polygon(w.pts, w.up_vector, w.normal) for w in shoebox_room_stub(*ROOM["dims"])]
    n = len(walls)
    patches = [kang.PatchesKang(w, ROOM["patch_size"], [j for j in range(n) if j != i], i,
                                scattering=ROOM["scattering"][i], absorption=ROOM["absorption"],
                                sound_attenuation_factor=ROOM["attenuation"]) for i, w in enumerate(walls)]
    radi = kang.RadiosityKang(patches, ROOM["patch_size"], ROOM["max_order_k"], ROOM["ir_length_s"],
                              speed_of_sound=ROOM["speed_of_sound"], sampling_rate=ROOM["sampling_rate"])
    source = so.SoundSource(ROOM["source"], [0, 1, 0], [0, 0, 1])
    radi.run(source)
    receiver = so.Receiver(ROOM["receiver"], [0, 1, 0], [0, 0, 1])
    out = {"room_ir": radi.energy_at_receiver(receiver), "room_ir_no_direct": radi.energy_at_receiver(
        receiver, ignore_direct=True), "room_ir_k2": radi.energy_at_receiver(receiver, max_order_k=2)}
    for i, p in enumerate(radi.patch_list):
        out[f"room_E_{i}"] = p.E_matrix
        out[f"room_ff_{i}"] = p.form_factors
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("SPARROWPY_SRC"),
                    help="sparrowpy source tree (default: $SPARROWPY_SRC)")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref or set SPARROWPY_SRC")
    out = stored_results(os.path.join(a.ref, "tests", "test_data"))
    out.update(reference_room(a.ref))
    out["room_config"] = np.array(json.dumps(ROOM))
    np.savez_compressed(os.path.join(HERE, "kang.npz"), **out)
    print("wrote", os.path.join(HERE, "kang.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
