"""CPU restatement of the Kang radiosity solver (test infrastructure only).

Follows sparrowpy/classes/RadiosityKang.py in FP64 with NumPy, per wall as
the reference does.  Used by tests/ to check the GPU path; pinned against
the reference's stored results and a run of the reference
(tests/golden/kang.npz, made by tests/golden/make_kang_golden.py).

A wall is a dict: pts (4, 3), normal (3,), max_size, other (wall ids),
scattering / absorption / attenuation (n_bins,), and after kang_patches its
patches (n, 4, 3).
"""
import numpy as np


def kang_patches(pts, max_size):
    """RadiosityKang.py:55-99: axis-aligned split of a wall into patches."""
    pts = np.asarray(pts, float)
    size = pts.max(axis=0) - pts.min(axis=0)
    nums = np.array([int(n) for n in size / max_size])
    with np.errstate(divide="ignore", invalid="ignore"):
        real = size / nums
    if nums[2] == 0:
        xi, yi = 0, 1
    if nums[1] == 0:
        xi, yi = 0, 2
    if nums[0] == 0:
        xi, yi = 1, 2
    x0, y0 = pts.T[xi].min(), pts.T[yi].min()
    out = []
    for ix in range(nums[xi]):
        for iy in range(nums[yi]):
            p = pts.copy()
            p[0, xi], p[0, yi] = x0 + ix * real[xi], y0 + iy * real[yi]
            p[1, xi], p[1, yi] = x0 + (ix + 1) * real[xi], y0 + iy * real[yi]
            p[3, xi], p[3, yi] = x0 + ix * real[xi], y0 + (iy + 1) * real[yi]
            p[2, xi], p[2, yi] = x0 + (ix + 1) * real[xi], y0 + (iy + 1) * real[yi]
            out.append(p)
    return np.array(out).reshape(-1, 4, 3)


def centers(p):
    return np.sum(p, axis=-2) / p.shape[-2]


def sizes(p):
    """geometry.py:84-89 `Polygon.size`."""
    return np.abs((p[..., 0, :] - p[..., 1, :]) - (p[..., 1, :] - p[..., 2, :]))


def init_energy(dl, dm, dn, dd_l, dd_m, sx, sy, sz, power, absorption, distance, attenuation):
    """RadiosityKang.py:812-849 `_init_energy_exchange` (one patch, all bands)."""
    half_l, half_m = dd_l / 2, dd_m / 2
    sin_phi_delta = (dl + half_l - sx) / np.sqrt(np.square(dl + half_l - sx) + np.square(dm - sy) + np.square(dn - sz))
    k_phi = -1 if (dl - half_l) <= sx and sx <= (dl + half_l) else 1
    sin_phi = k_phi * (dl - half_l - sx) / np.sqrt(np.square(dl - half_l - sx) + np.square(dm - sy) +
                                                   np.square(dn - sz))
    if (sin_phi_delta - sin_phi) < 1e-11:
        sin_phi *= -1
    plus = np.arctan(np.abs((dm + half_m - sy) / np.abs(sz)))
    minus = np.arctan(np.abs((dm - half_m - sy) / np.abs(sz)))
    k_beta = -1 if (dm - half_m) <= sy and sy <= (dm + half_m) else 1
    beta = np.abs(plus - (k_beta * minus))
    out = np.zeros(len(absorption))
    for b in range(len(absorption)):
        const = power * (1 - absorption[b]) * (np.exp(-attenuation[b] * distance))
        out[b] = const * (np.abs(sin_phi_delta - sin_phi)) * beta / (4 * np.pi)
    return out


def kang_init(wall, max_order, ir_length_s, src, power, fs, c):
    """RadiosityKang.py:141-207 `init_energy_exchange` for one wall: E (n_bins, K + 1, n, T)."""
    p = wall["patches"]
    nb = len(wall["absorption"])
    nt = int(ir_length_s * fs)
    E = np.zeros((nb, max_order + 1, p.shape[0], nt))
    nrm = np.asarray(wall["normal"], float)
    for i in range(p.shape[0]):
        s = np.asarray(src, float).copy()
        r = centers(p[i]).copy()
        distance = np.linalg.norm(r - s)
        delay = int(distance / c * fs)
        if np.abs(nrm[2]) > 0.99:
            ax, idx = 2, [0, 1, 2]
        elif np.abs(nrm[1]) > 0.99:
            ax, idx = 1, [2, 0, 1]
        elif np.abs(nrm[0]) > 0.99:
            ax, idx = 0, [1, 2, 0]
        else:
            raise AssertionError()
        off = r[ax]
        s[ax] = np.abs(s[ax] - off)
        r[ax] = np.abs(r[ax] - off)
        sz = sizes(p[i])
        E[:, 0, i, delay] += init_energy(r[idx[0]], r[idx[1]], r[idx[2]], sz[idx[0]], sz[idx[1]], s[idx[0]],
                                         s[idx[1]], s[idx[2]], power, wall["absorption"], distance,
                                         wall["attenuation"])
    return E


def _axes(n):
    if np.abs(n[0]) > 1e-5:
        return {2, 1}
    if np.abs(n[1]) > 1e-5:
        return {2, 0}
    if np.abs(n[2]) > 1e-5:
        return {0, 1}
    raise AssertionError()


def kang_ff(walls, w):
    """RadiosityKang.py:269-408 `calculate_form_factor` for wall w: (n_w, sum of the other walls' patches)."""
    me = walls[w]
    d = me["max_size"]
    cols = []
    for o in me["other"]:
        rw = walls[o]
        diff = np.abs(centers(rw["pts"]) - centers(me["pts"]))
        block = np.zeros((me["patches"].shape[0], rw["patches"].shape[0]))
        for i, sp in enumerate(me["patches"]):
            sc, sn = centers(sp), np.asarray(me["normal"], float)
            for j, rp in enumerate(rw["patches"]):
                rc, rn = centers(rp), np.asarray(rw["normal"], float)
                if np.dot(rn, sn) == 0:
                    i_s, i_r = _axes(sn), _axes(rn)
                    il = tuple(i_r.intersection(i_s))
                    i_ss = tuple(i_s.difference(set(il)))
                    i_rr = tuple(i_r.difference(set(il)))
                    dm = np.abs(sc[i_ss] - rc[i_ss])
                    dl, dlp = sc[il], rc[il]
                    dnp = np.abs(sc[i_rr] - rc[i_rr])
                    A = (dm - 0.5 * d) / np.sqrt((dl - dlp) ** 2 + (dm - 0.5 * d) ** 2 + dnp ** 2)
                    B = (dm + 0.5 * d) / np.sqrt(np.square(dl - dlp) + np.square(dm + 0.5 * d) + np.square(dnp))
                    one = np.arctan(np.abs((dl - 0.5 * d - dlp) / dnp))
                    two = np.arctan(np.abs((dl + 0.5 * d - dlp) / dnp))
                    k = -1 if np.abs(dl - dlp) < 1e-12 else 1
                    theta = np.abs(one - k * two)
                    ff = (1 / (2 * np.pi)) * np.abs(A ** 2 - B ** 2) * theta
                    ff = float(np.asarray(ff).reshape(-1)[0])
                else:
                    if diff[0] > 1e-5:
                        a, m_, b = 1, 0, 2
                    elif diff[1] > 1e-5:
                        a, m_, b = 0, 1, 2
                    elif diff[2] > 1e-5:
                        a, m_, b = 1, 2, 0
                    else:
                        raise AssertionError()
                    dist = np.sqrt((rc[a] - sc[a]) ** 2 + (rc[b] - sc[b]) ** 2 + (rc[m_] - sc[m_]) ** 2)
                    ff = (d * d * ((rc[m_] - sc[m_]) ** 2)) / (np.pi * dist ** 4)
                block[i, j] = ff
        cols.append(block)
    return np.concatenate(cols, axis=1) if cols else np.zeros((me["patches"].shape[0], 0))


def kang_exchange(walls, E, FF, w, k, c, fs):
    """RadiosityKang.py:209-267 `calculate_energy_exchange` for wall w, order k (updates E[w])."""
    me = walls[w]
    rc = centers(me["patches"])
    for r in range(rc.shape[0]):
        for o in me["other"]:
            sw = walls[o]
            col = sum(walls[x]["patches"].shape[0] for x in sw["other"][:list(sw["other"]).index(w)])
            sc = centers(sw["patches"])
            for s in range(sc.shape[0]):
                dist = np.linalg.norm(rc[r] - sc[s])
                delay = int(dist / c * fs)
                for b in range(len(me["absorption"])):
                    a_prev = E[o][b, k - 1, s, :]
                    if delay > a_prev.shape[-1]:
                        raise ValueError("delay longer than the histogram")
                    shifted = np.roll(a_prev, delay)
                    energy = shifted * FF[o][s, col + r] * me["scattering"][b] * (1 - me["absorption"][b]) * np.exp(
                        -me["attenuation"][b] * dist)
                    E[w][b, k, r, :] += energy


def kang_receiver(wall, E_w, max_order, rcv, c, fs):
    """RadiosityKang.py:443-498 `energy_at_receiver` of one wall: (n_bins, T)."""
    nb, _, n, nt = E_w.shape
    out = np.zeros((nb, nt))
    rcv = np.asarray(rcv, float)
    nrm = np.asarray(wall["normal"], float)
    for s, sp in enumerate(wall["patches"]):
        spos = centers(sp)
        diff = np.abs(rcv - spos)
        R = np.linalg.norm(spos - rcv)
        delay = int(R / c * fs)
        cos_xi = np.abs(np.sum(nrm * diff)) / np.linalg.norm(spos - rcv)
        for k in range(max_order + 1):
            for b in range(nb):
                factor = cos_xi * (np.exp(-wall["attenuation"][b] * R)) / (np.pi * R ** 2)
                out[b] += np.roll(E_w[b, k, s, :], delay) * factor
    return out


def kang_run(walls, max_order, ir_length_s, src, c, fs, power=1.0):
    """RadiosityKang.py:1005-1026 `run`: per wall E (n_bins, K + 1, n, T) and form factors."""
    E = [kang_init(w, max_order, ir_length_s, src, power, fs, c) for w in walls]
    FF = [kang_ff(walls, i) for i in range(len(walls))] if len(walls) > 1 else [None]
    if len(walls) > 1:
        for k in range(1, max_order + 1):
            for i in range(len(walls)):
                kang_exchange(walls, E, FF, i, k, c, fs)
    return E, FF


def kang_energy_at_receiver(walls, E, max_order, rcv, src, c, fs, ignore_direct=False):
    """RadiosityKang.py:1028-1046: the walls' responses plus the direct sound."""
    ir = 0
    for i, w in enumerate(walls):
        ir = ir + kang_receiver(w, E[i], max_order, rcv, c, fs)
    if not ignore_direct:
        m = np.asarray(walls[0]["attenuation"], float)
        r = np.sqrt(np.sum((np.asarray(rcv, float) - np.asarray(src, float)) ** 2))
        ir[:, int(r / c * fs)] += (1 / (4 * np.pi * np.square(r))) * np.exp(-m * r)
    return ir


def make_walls(polygons, max_size, scattering, absorption, attenuation):
    """Walls as RadiosityKang.py:945-955 builds them (every other wall visible)."""
    n = len(polygons)
    out = []
    for i, (pts, normal) in enumerate(polygons):
        out.append(dict(pts=np.asarray(pts, float), normal=np.asarray(normal, float), max_size=max_size,
                        other=[j for j in range(n) if j != i],
                        scattering=np.atleast_1d(np.asarray(scattering[i], float)),
                        absorption=np.atleast_1d(np.asarray(absorption, float)),
                        attenuation=np.atleast_1d(np.asarray(attenuation, float)),
                        patches=kang_patches(pts, max_size)))
    return out


# ------------------------------------------------------------- directional variant
# A directional wall adds: dir_data (n_src_dirs, n_dirs, n_bins) (already |data| * pi),
# dir_sources (n_src_dirs, 3) and dir_receivers (n_dirs, 3), both in the wall's frame
# (reference_frame_directions).

def wall_frame_directions(xyz, normal, up):
    """RadiosityKang.py:558-567: directions of the data frame (normal +z, up +x) in the wall's frame, radius 1.

    Restated with the rotation matrix whose columns are (up, normal x up, normal), not through Euler angles."""
    n = np.asarray(normal, float) / np.linalg.norm(normal)
    u = np.asarray(up, float) / np.linalg.norm(up)
    rot = np.stack([u, np.cross(n, u), n], axis=1)
    out = np.asarray(xyz, float).reshape(-1, 3) @ rot.T
    return out / np.linalg.norm(out, axis=1)[:, None]


def reference_frame_directions(xyz, normal, up):
    """RadiosityKang.py:558-567 step by step, with scipy's Rotation (pyfar's Orientations extend it).

    o1 = from_view_up(normal, up) and o2 = from_view_up(+z, +x) are the rotations whose matrix rows are
    (view, up, view x up); the directions are rotated by the 'xyz' Euler angles (degrees) of o1^-1 o2 and
    moved to radius 1 through spherical coordinates (azimuth = atan2(y, x) mod 2 pi, colatitude =
    arccos(z / r); back with x = (r sin col) cos az, y = (r sin col) sin az, z = r cos col, components
    below the FP64 epsilon set to 0), as pyfar's Coordinates.rotate and radius assignment do.  Ties of
    the nearest-direction search depend on these roundings."""
    import warnings
    from scipy.spatial.transform import Rotation

    def orientation(view, upv):
        view = np.asarray(view, float) / np.linalg.norm(view)
        upv = np.asarray(upv, float) / np.linalg.norm(upv)
        return Rotation.from_matrix(np.stack([view, upv, np.cross(view, upv)])[None])

    with warnings.catch_warnings():
        warnings.simplefilter("ignore", UserWarning)
        euler = (orientation(normal, up).inv() * orientation([0, 0, 1], [1, 0, 0])).as_euler('xyz', True).flatten()
    p = Rotation.from_euler('xyz', euler, degrees=True).apply(np.asarray(xyz, float).reshape(-1, 3))
    return unit_sphere(p)


def unit_sphere(p):
    """Points moved to radius 1 through spherical coordinates, as pyfar's `radius = 1` does."""
    p = np.asarray(p, float).reshape(-1, 3)
    r = np.sqrt(p[:, 0] ** 2 + p[:, 1] ** 2 + p[:, 2] ** 2)
    az = np.mod(np.arctan2(p[:, 1], p[:, 0]), 2 * np.pi)
    col = np.arccos(np.divide(p[:, 2], r, out=np.zeros_like(r), where=r != 0))
    rs = 1.0 * np.sin(col)
    out = np.stack([rs * np.cos(az), rs * np.sin(az), 1.0 * np.cos(col)], axis=1)
    out[np.abs(out) < np.finfo(float).eps] = 0
    return out


def nearest(points, q):
    """Index of the nearest point of every query: a k-d tree on the Euclidean distance, as pyfar's
    Coordinates.find_nearest (scipy's cKDTree), so that exact ties resolve as in the reference."""
    from scipy.spatial import cKDTree
    return cKDTree(np.asarray(points, float).reshape(-1, 3)).query(np.asarray(q, float).reshape(-1, 3))[1]


def dkang_init(wall, max_order, ir_length_s, src, power, fs, c):
    """RadiosityKang.py:629-671: the plain init tiled over the outgoing directions, times |data| of the
    source direction nearest to (source - patch centre)."""
    E = kang_init(wall, max_order, ir_length_s, src, power, fs, c)
    nd = wall["dir_data"].shape[1]
    E = np.repeat(E[..., None], nd, axis=-1)
    ctr = centers(wall["patches"])
    idx = nearest(wall["dir_sources"], np.asarray(src, float)[None, :] - ctr)
    for b in range(E.shape[0]):
        for i in range(ctr.shape[0]):
            E[b, 0, i, :, :] *= np.abs(wall["dir_data"][idx[i], :, b])
    return E


def dkang_exchange(walls, E, FF, w, k, c, fs):
    """RadiosityKang.py:673-745 for wall w, order k: per (receiver, source) the delayed source histograms
    (every outgoing direction) times ff (1 - alpha) exp(-m d), times the receiver wall's data row of the
    source direction nearest to (source centre - receiver centre)."""
    me = walls[w]
    rc = centers(me["patches"])
    for r in range(rc.shape[0]):
        for o in me["other"]:
            sw = walls[o]
            col = sum(walls[x]["patches"].shape[0] for x in sw["other"][:list(sw["other"]).index(w)])
            sc = centers(sw["patches"])
            for s in range(sc.shape[0]):
                dist = np.linalg.norm(rc[r] - sc[s])
                delay = int(dist / c * fs)
                ff = FF[o][s, col + r]
                for b in range(len(me["absorption"])):
                    a_prev = E[o][b, k - 1, s, :, :]
                    if delay > a_prev.shape[0]:
                        raise ValueError("delay longer than the histogram")
                    energy = np.roll(a_prev, delay, axis=0) * ff * (1 - me["absorption"][b]) * np.exp(
                        -me["attenuation"][b] * dist)
                    idx = nearest(me["dir_sources"], sc[s] - rc[r])[0]
                    energy *= me["dir_data"][idx, :, b]
                    E[w][b, k, r, :, :] += energy


def dkang_receiver(wall, E_w, max_order, rcv, c, fs):
    """RadiosityKang.py:747-810: each patch's histogram of the outgoing direction nearest to the receiver."""
    nb, _, n, nt, _ = E_w.shape
    out = np.zeros((nb, nt))
    rcv = np.asarray(rcv, float)
    nrm = np.asarray(wall["normal"], float)
    for s, sp in enumerate(wall["patches"]):
        spos = centers(sp)
        cos_xi = np.abs(np.sum(nrm * np.abs(rcv - spos))) / np.linalg.norm(spos - rcv)
        i_dir = nearest(wall["dir_receivers"], unit_sphere(rcv - spos))[0]
        R = np.linalg.norm(rcv - spos)
        delay = int(R / c * fs)
        for k in range(max_order + 1):
            for b in range(nb):
                factor = cos_xi * (np.exp(-wall["attenuation"][b] * R)) / (np.pi * R ** 2)
                out[b] += np.roll(E_w[b, k, s, :, i_dir], delay) * factor
    return out


def dkang_run(walls, max_order, ir_length_s, src, c, fs, power=1.0):
    """RadiosityKang.py:1163-1184 over directional walls: per wall E (n_bins, K + 1, n, T, n_dirs)."""
    E = [dkang_init(w, max_order, ir_length_s, src, power, fs, c) for w in walls]
    FF = [kang_ff(walls, i) for i in range(len(walls))] if len(walls) > 1 else [None]
    if len(walls) > 1:
        for k in range(1, max_order + 1):
            for i in range(len(walls)):
                dkang_exchange(walls, E, FF, i, k, c, fs)
    return E, FF


def dkang_energy_at_receiver(walls, E, max_order, rcv, src, c, fs):
    """RadiosityKang.py:1186-1202: the walls' responses plus the direct sound."""
    ir = 0
    for i, w in enumerate(walls):
        ir = ir + dkang_receiver(w, E[i], max_order, rcv, c, fs)
    m = np.asarray(walls[0]["attenuation"], float)
    r = np.sqrt(np.sum((np.asarray(rcv, float) - np.asarray(src, float)) ** 2))
    ir[:, int(r / c * fs)] += (1 / (4 * np.pi * np.square(r))) * np.exp(-m * r)
    return ir
