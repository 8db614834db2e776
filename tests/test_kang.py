"""Kang radiosity (sparrowpy/classes/RadiosityKang.py; tests/test_Radiosity.py).

Golden vectors (tests/golden/kang.npz) hold the reference's own stored
results and a run of the reference here (make_kang_golden.py).  The CPU
tests pin the oracle (oracle/kang.py) to them; the GPU tests run
sparrowpy_gb300.kang (CUDA, FP64) against the same vectors and against the
oracle.  The reference compares its stored results to 2-7 decimals; the
restatements here agree to 1e-12 relative where the arithmetic is the
reference's (the FP64 library functions exp and arctan may differ in the
last bit).
"""
import json
import os

import numpy as np
import numpy.testing as npt
import pytest

from oracle import kang as ok
from sparrowpy_gb300.geometry import shoebox_room_stub

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "kang.npz"))
ROOM = json.loads(str(GOLD["room_config"]))  # written by make_kang_golden.py
PARALLEL = [[0, 1], [1, 0], [2, 3], [3, 2], [4, 5], [5, 4]]
PERPENDICULAR = [[i, j] for i in range(6) for j in range(6) if i // 2 != j // 2]


def cube_pair(i, j, size):
    """Two unit-cube walls as the reference's tests build them: PatchesKang(w_i, size, [1], 0), (w_j, size, [0], 1)."""
    walls = shoebox_room_stub(1, 1, 1)
    out = []
    for k, (w, other) in enumerate(((walls[i], [1]), (walls[j], [0]))):
        out.append(dict(pts=np.asarray(w.pts, float), normal=np.asarray(w.normal, float), max_size=size, other=other,
                        scattering=np.ones(1), absorption=np.full(1, 0.1), attenuation=np.zeros(1),
                        patches=ok.kang_patches(w.pts, size)))
    return out


def room_walls():
    walls = shoebox_room_stub(*ROOM["dims"])
    return ok.make_walls([(w.pts, w.normal) for w in walls], ROOM["patch_size"], ROOM["scattering"],
                         ROOM["absorption"], ROOM["attenuation"])


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


@pytest.mark.parametrize("size", [0.5, 1])
@pytest.mark.parametrize("pair", PARALLEL)
def test_oracle_ff_parallel(pair, size):
    walls = cube_pair(*pair, size)
    npt.assert_allclose(ok.kang_ff(walls, 0), GOLD[f"ff_parallel_size{size:g}"], rtol=1e-12)


@pytest.mark.parametrize("pair", PERPENDICULAR)
def test_oracle_ff_perpendicular(pair):
    npt.assert_allclose(ok.kang_ff(cube_pair(*pair, 0.5), 0), GOLD[f"ff_perpendicular_{pair[0]}_{pair[1]}_size0.5"],
                        rtol=1e-12)
    ff = np.sort(ok.kang_ff(cube_pair(*pair, 0.5), 0).reshape(-1))
    npt.assert_allclose(ff, GOLD["ff_perpendicular_sorted_size0.5"], rtol=1e-12)
    npt.assert_allclose(ok.kang_ff(cube_pair(*pair, 1), 0), GOLD["ff_perpendicular_0_0_size1"], rtol=1e-12)


@pytest.mark.parametrize("size", [0.5, 1])
@pytest.mark.parametrize("wall", range(6))
def test_oracle_init_energy(wall, size):
    w = cube_pair(wall, wall, size)[0]
    E = ok.kang_init(w, 3, 5, [0.5, 0.5, 0.5], 1.0, 1000, 346.18)
    npt.assert_allclose(E, GOLD[f"E_init_size{size:g}"], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("size", [0.5, 1])
def test_oracle_energy_exchange(size):
    walls = cube_pair(0, 2, size)
    E = [ok.kang_init(w, 3, 5, [0.5, 0.5, 0.5], 1.0, 1000, 346.18) for w in walls]
    FF = [ok.kang_ff(walls, 0), ok.kang_ff(walls, 1)]
    for k in range(1, 4):
        ok.kang_exchange(walls, E, FF, 0, k, 346.18, 1000)
        ok.kang_exchange(walls, E, FF, 1, k, 346.18, 1000)
    npt.assert_allclose(E[0], GOLD[f"E_exchange_size{size:g}"], rtol=1e-12, atol=1e-300)


def test_oracle_room_matches_reference_run():
    walls = room_walls()
    E, FF = ok.kang_run(walls, ROOM["max_order_k"], ROOM["ir_length_s"], ROOM["source"], ROOM["speed_of_sound"],
                        ROOM["sampling_rate"])
    for i in range(6):
        npt.assert_allclose(FF[i], GOLD[f"room_ff_{i}"], rtol=1e-12, atol=1e-300)
        assert rel(E[i], GOLD[f"room_E_{i}"]) < 1e-12
    args = (walls, E, ROOM["max_order_k"], ROOM["receiver"], ROOM["source"], ROOM["speed_of_sound"],
            ROOM["sampling_rate"])
    assert rel(ok.kang_energy_at_receiver(*args), GOLD["room_ir"]) < 1e-12
    assert rel(ok.kang_energy_at_receiver(*args, ignore_direct=True), GOLD["room_ir_no_direct"]) < 1e-12
    args2 = (walls, E, 2) + args[3:]
    assert rel(ok.kang_energy_at_receiver(*args2), GOLD["room_ir_k2"]) < 1e-12


def x10_walls():
    """The reference's 10 x 20 x 15 m ground + two facades (test_Radiosity.py:236-283)."""
    X, Y, Z = 10, 20, 15
    polys = [([[0, 0, 0], [X, 0, 0], [X, Y, 0], [0, Y, 0]], [0, 0, 1]),
             ([[0, 0, 0], [X, 0, 0], [X, 0, Z], [0, 0, Z]], [0, 1, 0]),
             ([[0, Y, 0], [X, Y, 0], [X, Y, Z], [0, Y, Z]], [0, -1, 0])]
    return ok.make_walls(polys, 5, [1.0, 1.0, 1.0], [0.1], [0.0])


@pytest.mark.parametrize("k", [2, 3])
def test_oracle_x10_simulation(k):
    walls = x10_walls()
    E, _ = ok.kang_run(walls, k, 5, [10, 6, 1], 343, 50)
    ir = ok.kang_energy_at_receiver(walls, E, k, [20, 2, 1], [10, 6, 1], 343, 50)
    ir = ir / np.max(np.abs(ir))
    npt.assert_almost_equal(GOLD[f"sim_X10_k{k}_time"][0], ir[0], decimal=2)


# ------------------------------------------------------------- host, no GPU
def test_kang_objects_round_trip(tmp_path):
    import sparrowpy_gb300 as sp
    walls = shoebox_room_stub(2, 1, 1)
    radi = sp.RadiosityKang(walls, 0.5, 3, 0.1, speed_of_sound=343, sampling_rate=1000, absorption=0.2)
    assert [len(p.patches) for p in radi.patch_list] == [8, 8, 8, 8, 4, 4]
    npt.assert_array_equal(radi.patch_list[0].other_wall_ids, [1, 2, 3, 4, 5])
    d = radi.to_dict()
    back = sp.RadiosityKang.from_dict(dict(d, source_position=None))
    assert back.patch_size == 0.5 and back.max_order_k == 3 and len(back.patch_list) == 6
    npt.assert_array_equal(back.patch_list[2].pts, radi.patch_list[2].pts)
    npt.assert_array_equal(back.patch_list[2].absorption, [0.2])
    radi.write(tmp_path / "kang.far")
    read = sp.RadiosityKang.from_read(tmp_path / "kang.far")
    assert read.ir_length_s == 0.1 and read.sampling_rate == 1000
    for a, b in zip(read.patch_list, radi.patch_list):
        npt.assert_array_equal(a.pts, b.pts)
        npt.assert_array_equal(a.other_wall_ids, b.other_wall_ids)
        assert a.wall_id == b.wall_id and a.E_matrix is None


# ------------------------------------------------------------------- GPU
def gpu_pair(i, j, size):
    import sparrowpy_gb300 as sp
    walls = shoebox_room_stub(1, 1, 1)
    return sp.PatchesKang(walls[i], size, [1], 0), sp.PatchesKang(walls[j], size, [0], 1)


@pytest.mark.gpu
@pytest.mark.parametrize("size", [0.5, 1])
def test_gpu_ff_parallel(size):
    for pair in PARALLEL:
        p1, p2 = gpu_pair(*pair, size)
        p1.calculate_form_factor([p1, p2])
        npt.assert_allclose(p1.form_factors, GOLD[f"ff_parallel_size{size:g}"], rtol=1e-12)


@pytest.mark.gpu
def test_gpu_ff_perpendicular():
    for pair in PERPENDICULAR:
        p1, p2 = gpu_pair(*pair, 0.5)
        p1.calculate_form_factor([p1, p2])
        npt.assert_allclose(p1.form_factors, GOLD[f"ff_perpendicular_{pair[0]}_{pair[1]}_size0.5"], rtol=1e-12)
        p1, p2 = gpu_pair(*pair, 1)
        p1.calculate_form_factor([p1, p2])
        npt.assert_allclose(p1.form_factors, GOLD["ff_perpendicular_0_0_size1"], rtol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("size", [0.5, 1])
def test_gpu_init_energy(size):
    from sparrowpy_gb300.sound_object import SoundSource
    source = SoundSource([0.5, 0.5, 0.5], [0, 1, 0], [0, 0, 1])
    for wall in range(6):
        p = gpu_pair(wall, wall, size)[0]
        p.init_energy_exchange(3, 5, source, 1000, 346.18)
        npt.assert_allclose(p.E_matrix, GOLD[f"E_init_size{size:g}"], rtol=1e-12, atol=1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("size", [0.5, 1])
@pytest.mark.parametrize("pair", [[0, 2], [2, 0]])
def test_gpu_energy_exchange(pair, size):
    """As the reference's test_energy_exchange; [0, 2] is the stored case itself, [2, 0] its mirror."""
    from sparrowpy_gb300.sound_object import SoundSource
    p1, p2 = gpu_pair(*pair, size)
    source = SoundSource([0.5, 0.5, 0.5], [0, 1, 0], [0, 0, 1])
    patches = [p1, p2]
    p1.calculate_form_factor(patches)
    p2.calculate_form_factor(patches)
    p1.init_energy_exchange(3, 5, source, 1000, 346.18)
    p2.init_energy_exchange(3, 5, source, 1000, 346.18)
    for k in range(1, 4):
        p1.calculate_energy_exchange(patches, k, speed_of_sound=346.18, E_sampling_rate=1000)
        p2.calculate_energy_exchange(patches, k, speed_of_sound=346.18, E_sampling_rate=1000)
    gold = GOLD[f"E_exchange_size{size:g}"]
    if pair == [0, 2]:
        npt.assert_allclose(p1.E_matrix, gold, rtol=1e-12, atol=1e-300)
    else:  # the reference's own tolerance for the mirrored case
        with np.errstate(divide="ignore"):
            npt.assert_almost_equal(10 * np.log10(gold), 10 * np.log10(p1.E_matrix), decimal=1)
    # and against the oracle on the same walls
    walls = cube_pair(*pair, size)
    E = [ok.kang_init(w, 3, 5, [0.5, 0.5, 0.5], 1.0, 1000, 346.18) for w in walls]
    FF = [ok.kang_ff(walls, 0), ok.kang_ff(walls, 1)]
    for k in range(1, 4):
        ok.kang_exchange(walls, E, FF, 0, k, 346.18, 1000)
        ok.kang_exchange(walls, E, FF, 1, k, 346.18, 1000)
    npt.assert_allclose(p1.E_matrix, E[0], rtol=1e-12, atol=1e-300)
    npt.assert_allclose(p2.E_matrix, E[1], rtol=1e-12, atol=1e-300)


@pytest.mark.gpu
def test_gpu_room_matches_reference_run():
    import sparrowpy_gb300 as sp
    from sparrowpy_gb300.sound_object import Receiver, SoundSource
    walls = shoebox_room_stub(*ROOM["dims"])
    n = len(walls)
    patches = [sp.PatchesKang(w, ROOM["patch_size"], [j for j in range(n) if j != i], i,
                              scattering=ROOM["scattering"][i], absorption=ROOM["absorption"],
                              sound_attenuation_factor=ROOM["attenuation"]) for i, w in enumerate(walls)]
    radi = sp.RadiosityKang(patches, ROOM["patch_size"], ROOM["max_order_k"], ROOM["ir_length_s"],
                            speed_of_sound=ROOM["speed_of_sound"], sampling_rate=ROOM["sampling_rate"])
    radi.run(SoundSource(ROOM["source"], [0, 1, 0], [0, 0, 1]))
    for i, p in enumerate(radi.patch_list):
        npt.assert_allclose(p.form_factors, GOLD[f"room_ff_{i}"], rtol=1e-12, atol=1e-300)
        assert rel(p.E_matrix, GOLD[f"room_E_{i}"]) < 1e-12
    rcv = Receiver(ROOM["receiver"], [0, 1, 0], [0, 0, 1])
    assert rel(radi.energy_at_receiver(rcv), GOLD["room_ir"]) < 1e-12
    assert rel(radi.energy_at_receiver(rcv, ignore_direct=True), GOLD["room_ir_no_direct"]) < 1e-12
    assert rel(radi.energy_at_receiver(rcv, max_order_k=2), GOLD["room_ir_k2"]) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("k", [2, 3])
def test_gpu_x10_simulation(k):
    """The reference's test_radiosity_reference (test_Radiosity.py:236-283) with its tolerance."""
    import sparrowpy_gb300 as sp
    from sparrowpy_gb300.geometry import Polygon
    from sparrowpy_gb300.sound_object import Receiver, SoundSource
    X, Y, Z = 10, 20, 15
    ground = Polygon([[0, 0, 0], [X, 0, 0], [X, Y, 0], [0, Y, 0]], [1, 0, 0], [0, 0, 1])
    a_wall = Polygon([[0, 0, 0], [X, 0, 0], [X, 0, Z], [0, 0, Z]], [1, 0, 0], [0, 1, 0])
    b_wall = Polygon([[0, Y, 0], [X, Y, 0], [X, Y, Z], [0, Y, Z]], [1, 0, 0], [0, -1, 0])
    radi = sp.RadiosityKang([ground, a_wall, b_wall], 5, k, 5, speed_of_sound=343, sampling_rate=50)
    radi.run(SoundSource([10, 6, 1], [0, 1, 0], [0, 0, 1]))
    ir = radi.energy_at_receiver(Receiver([20, 2, 1], [0, 1, 0], [0, 0, 1]))
    ir = ir / np.max(np.abs(ir))
    npt.assert_almost_equal(GOLD[f"sim_X{X}_k{k}_time"][0], ir[0], decimal=2)
    # and the oracle, tightly
    walls = x10_walls()
    E, _ = ok.kang_run(walls, k, 5, [10, 6, 1], 343, 50)
    ref = ok.kang_energy_at_receiver(walls, E, k, [20, 2, 1], [10, 6, 1], 343, 50)
    assert rel(ir, ref / np.max(np.abs(ref))) < 1e-12


@pytest.mark.gpu
def test_gpu_source_delay_past_histogram_raises():
    """A source farther than the histogram reaches: the reference's E_matrix indexing raises IndexError."""
    import sparrowpy_gb300 as sp
    from sparrowpy_gb300.sound_object import SoundSource
    p = sp.PatchesKang(shoebox_room_stub(1, 1, 1)[0], 0.5, [], 0)
    with pytest.raises(IndexError):
        p.init_energy_exchange(1, 0.01, SoundSource([0.5, 100.0, 0.5], [0, 1, 0], [0, 0, 1]), 1000, 343.0)


# ------------------------------------------------ the reference's properties
def _kang_room(dims, patch_size, max_order, src, sampling_rate=1, ir_length_s=1, shift=(0.0, 0.0, 0.0)):
    import sparrowpy_gb300 as sp
    from sparrowpy_gb300.geometry import SoundSource
    walls = shoebox_room_stub(*dims)
    for w in walls:
        w.pts += np.asarray(shift)
    radi = sp.RadiosityKang(walls, patch_size, max_order, ir_length_s, speed_of_sound=343,
                            sampling_rate=sampling_rate, absorption=0.1)
    radi.run(SoundSource(np.asarray(src, float) + np.asarray(shift), [0, 1, 0], [0, 0, 1]))
    return radi


@pytest.mark.gpu
def test_gpu_small_room_and_shift():
    """test_Radiosity.py:16-80: a shifted room gives identical E_matrix, form factors and response."""
    from sparrowpy_gb300.geometry import Receiver
    out = []
    for shift in ((0.0, 0.0, 0.0), (2.0, 4.0, 5.0)):
        radi = _kang_room((5, 6, 4), 1, 10, [2, 2, 2], shift=shift)
        E = np.concatenate([p.E_matrix for p in radi.patch_list], axis=-2)
        ff = [p.form_factors for p in radi.patch_list]
        ir = radi.energy_at_receiver(Receiver(np.array([3.0, 2.0, 3.0]) + shift, [0, 1, 0], [0, 0, 1]),
                                     ignore_direct=True)
        out.append((E, ff, ir))
    npt.assert_array_equal(out[0][0], out[1][0])
    for a, b in zip(out[0][1], out[1][1]):
        npt.assert_array_equal(a, b)
    npt.assert_array_equal(out[0][2], out[1][2])


@pytest.mark.gpu
def test_gpu_small_room_and_rotate():
    """test_Radiosity.py:82-141: the six axis permutations of a room give the same response (4 decimals)."""
    from sparrowpy_gb300.geometry import Receiver
    X, Y, Z = 5, 3, 4
    r = (1, 2, 1.5)
    perms = [(0, 1, 2), (0, 2, 1), (1, 2, 0), (1, 0, 2), (2, 0, 1), (2, 1, 0)]
    irs = []
    for p in perms:
        dims = [(X, Y, Z)[k] for k in p]
        radi = _kang_room(dims, 1, 10, [2, 2, 2])
        irs.append(radi.energy_at_receiver(Receiver([r[k] for k in p], [0, 1, 0], [0, 0, 1]),
                                           ignore_direct=True).squeeze())
    irs = np.array(irs)
    npt.assert_array_almost_equal(irs, irs[0], decimal=4)


@pytest.mark.gpu
@pytest.mark.parametrize("patch_size", [1, 0.5, 0.2, 1 / 3])
def test_gpu_init_energy_larger_0(patch_size):
    """test_Radiosity.py:635-660: a cube's patches receive energy from a central source (and match the oracle)."""
    import sparrowpy_gb300 as sp
    from sparrowpy_gb300.geometry import SoundSource
    radi = sp.RadiosityKang(shoebox_room_stub(1, 1, 1), patch_size, 0, 1, speed_of_sound=343, sampling_rate=1,
                            absorption=0.1)
    source = SoundSource([0.5, 0.5, 0.5], [0, 1, 0], [0, 0, 1])
    for p in radi.patch_list:
        p.init_energy_exchange(radi.max_order_k, radi.ir_length_s, source, sampling_rate=radi.sampling_rate,
                               speed_of_sound=343)
    E = np.concatenate([p.E_matrix for p in radi.patch_list], axis=-2)
    assert E.flatten()[0] > 0
    walls = ok.make_walls([(w.pts, w.normal) for w in shoebox_room_stub(1, 1, 1)], patch_size, [1.0] * 6, [0.1],
                          [0.0])
    ref = np.concatenate([ok.kang_init(w, 0, 1, [0.5, 0.5, 0.5], 1.0, 1, 343) for w in walls], axis=-2)
    npt.assert_allclose(E, ref, rtol=1e-12, atol=1e-300)
