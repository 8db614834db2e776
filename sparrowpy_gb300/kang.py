"""The Kang radiosity solver (sparrowpy/classes/RadiosityKang.py) on the GPU, FP64.

PatchesKang is a wall split into patches with its energy matrix E_matrix
(n_bins, max_order + 1, n_patches, n_samples) and form factors towards the
other walls' patches; RadiosityKang runs every wall (run) and collects the
energy at a receiver.  Each step is one C-ABI call on the wall's device
arrays (csrc/kang.cu):

* init_energy_exchange: the closed-form source energy of every patch
  (RadiosityKang.py:141-207, :812-849);
* calculate_form_factor: the closed forms for parallel and perpendicular
  patches (:269-408);
* calculate_energy_exchange: one call per source wall, in the wall's order
  (:209-267), so every histogram bin sums its terms in the reference's
  order;
* energy_at_receiver: per wall (:443-498), plus the direct sound
  (:1028-1046) on the host.

E_matrix and form_factors read back to NumPy on access.

The directional variant (PatchesDirectionalKang, DirectionalRadiosityKang,
RadiosityKang.py:500-810 and :1059-1202) keeps one histogram per outgoing
direction of the wall's directional data (n_src_dirs, n_dirs, n_bins): the
source energy and every exchanged term are weighted by the data row of the
source direction nearest to the incoming direction, and a receiver reads
the row of the outgoing direction nearest to it.  The data is read from
SOFA files (sofa.py) or given as arrays, and rotated into the wall's frame
as pyfar's Orientations and Coordinates.rotate do (scipy's Rotation, which
pyfar's Orientations extends).  Nearest directions are found with scipy's
cKDTree on the host, as pyfar's find_nearest does; the sums run on the
same kernels as the plain solver, templated on the direction axis.
"""
import ctypes
import warnings

import numpy as np
import torch

from . import _native as nat
from . import far
from .coords import Coordinates, FrequencyData, unit_radius
from .geometry import Polygon, create_patches
from .sound_object import SoundSource


def _ptr(t):
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dev(a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def _sizes(pts):
    """geometry.py:84-89 `Polygon.size` of each patch: |(p0 - p1) - (p1 - p2)|."""
    return np.abs((pts[:, 0] - pts[:, 1]) - (pts[:, 1] - pts[:, 2]))


def _raise_for(err, what):
    code = int(err.item())
    if code == 1:
        raise IndexError(f"{what}: a source delay falls outside the energy histogram")
    if code == 2:
        raise ValueError(f"{what}: a delay is longer than the energy histogram")


class PatchesKang(Polygon):
    """A wall split into patches (RadiosityKang.py:9-105)."""

    def __init__(self, polygon, max_size, other_wall_ids, wall_id, scattering=1, absorption=0.1,
                 sound_attenuation_factor=0, E_matrix=None):
        Polygon.__init__(self, polygon.pts, polygon.up_vector, polygon.normal)
        self.scattering = np.atleast_1d(np.asarray(scattering, dtype=float))
        self.absorption = np.atleast_1d(np.asarray(absorption, dtype=float))
        self.sound_attenuation_factor = np.atleast_1d(np.asarray(sound_attenuation_factor, dtype=float))
        assert self.scattering.size == self.absorption.size
        assert self.scattering.size == self.sound_attenuation_factor.size
        self.n_bins = self.absorption.size
        with np.errstate(divide="ignore", invalid="ignore"):
            pts = create_patches(self.pts, max_size)
        self.patches = [Polygon(p, polygon.up_vector, polygon.normal) for p in pts]
        self._pts = pts
        self.other_wall_ids = np.atleast_1d(np.array(other_wall_ids, dtype=int))
        self.wall_id = wall_id
        self.max_size = max_size
        self._E = None
        self._ff = None
        self._g = None
        if E_matrix is not None:
            self.E_matrix = E_matrix

    # ------------------------------------------------------------ device data
    def _geometry(self):
        if self._g is None:
            ctr = np.sum(self._pts, axis=1) / self._pts.shape[1]
            self._g = dict(centers=_dev(ctr.reshape(-1, 3)), sizes=_dev(_sizes(self._pts).reshape(-1, 3)),
                           normal=_dev(self.normal))
        # the material arrays are read at every call, as the reference reads its attributes
        return dict(self._g, scattering=_dev(self.scattering), absorption=_dev(self.absorption),
                    attenuation=_dev(self.sound_attenuation_factor))

    @property
    def E_matrix(self):
        """The energy matrix (n_bins, max_order + 1, n_patches, n_samples)."""
        return None if self._E is None else self._E.cpu().numpy()

    @E_matrix.setter
    def E_matrix(self, value):
        self._E = _dev(value) if value is not None else None
        if value is not None:
            self.E_n_samples = int(np.shape(value)[3])

    @property
    def form_factors(self):
        """Form factors (n_patches, patches of the other walls, in other_wall_ids order)."""
        return None if self._ff is None else self._ff.cpu().numpy()

    # ---------------------------------------------------------------- steps
    def init_energy_exchange(self, max_order_k, ir_length_s, source, sampling_rate, speed_of_sound):
        """Source energy of every patch at its delay, order 0 (RadiosityKang.py:141-207)."""
        self.E_sampling_rate = sampling_rate
        self.E_n_samples = int(ir_length_s * sampling_rate)
        n = len(self.patches)
        nrm = np.abs(np.asarray(self.normal, dtype=float))
        if not (nrm[2] > 0.99 or nrm[1] > 0.99 or nrm[0] > 0.99):
            raise AssertionError()
        self._E = torch.zeros((self.n_bins, max_order_k + 1, n, self.E_n_samples), dtype=torch.float64,
                              device="cuda")
        if n == 0 or self.E_n_samples == 0:
            return
        g = self._geometry()
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        src = _dev(np.asarray(source.position, dtype=float).reshape(3))
        nat.call("sp_kang_init_energy", n, _ptr(g["centers"]), _ptr(g["sizes"]), _ptr(g["normal"]), _ptr(src),
                 float(source.sound_power), self.n_bins, _ptr(g["absorption"]), _ptr(g["attenuation"]),
                 float(speed_of_sound), float(sampling_rate), max_order_k + 1, self.E_n_samples, _ptr(self._E),
                 _ptr(err), _stream())
        _raise_for(err, "init_energy_exchange")

    def calculate_form_factor(self, patches_list):
        """Form factors towards the other walls' patches (RadiosityKang.py:269-408)."""
        n = len(self.patches)
        cols_c, cols_n, cols_w = [], [], []
        for wid in self.other_wall_ids:
            wall = patches_list[wid]
            m = len(wall.patches)
            ctr = np.sum(wall._pts, axis=1) / wall._pts.shape[1]
            cols_c.append(ctr.reshape(-1, 3))
            cols_n.append(np.tile(np.asarray(wall.normal, float), (m, 1)))
            cols_w.append(np.tile(np.asarray(wall.center, float), (m, 1)))
            parallel = np.dot(np.asarray(wall.normal, float), np.asarray(self.normal, float)) != 0
            if parallel and m and n and not np.any(np.abs(np.asarray(wall.center) - np.asarray(self.center)) > 1e-5):
                raise AssertionError()
        n_r = int(sum(c.shape[0] for c in cols_c))
        self._ff = torch.zeros((n, n_r), dtype=torch.float64, device="cuda")
        if n == 0 or n_r == 0:
            return
        g = self._geometry()
        rc, rn, rw = (_dev(np.concatenate(x)) for x in (cols_c, cols_n, cols_w))
        wc = _dev(self.center)  # held until the call has been enqueued and the result read
        nat.call("sp_kang_form_factors", n, _ptr(g["centers"]), _ptr(g["normal"]), _ptr(wc), n_r,
                 _ptr(rc), _ptr(rn), _ptr(rw), float(self.max_size), _ptr(self._ff), _stream())

    def get_form_factor(self, patches_list, source_path_id, receiver_wall_id, receiver_patch_id):
        """One form factor (RadiosityKang.py:410-441)."""
        return self.form_factors[source_path_id, self._column(patches_list, receiver_wall_id) + receiver_patch_id]

    def _column(self, patches_list, wall_id):
        off = 0
        for other in self.other_wall_ids:
            if other == wall_id:
                return off
            off += len(patches_list[other].patches)
        raise KeyError(f"wall {wall_id} is not among this wall's other walls")

    def calculate_energy_exchange(self, patches_list, current_order_k, speed_of_sound, E_sampling_rate):
        """Order k of this wall from the other walls' order k - 1 (RadiosityKang.py:209-267)."""
        k = current_order_k
        n = len(self.patches)
        nb, n_orders, _, nt = self._E.shape
        g = self._geometry()
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        for wid in self.other_wall_ids:
            wall = patches_list[wid]
            m = len(wall.patches)
            if n == 0 or m == 0:
                continue
            col0 = wall._column(patches_list, self.wall_id)
            wsz = nat.size("sp_kang_exchange_workspace", n, m, nb)
            ws = torch.empty((wsz,), dtype=torch.uint8, device="cuda")
            wg = wall._geometry()
            nat.call("sp_kang_exchange", k, nb, n_orders, nt, n, _ptr(g["centers"]), _ptr(self._E),
                     _ptr(g["scattering"]), _ptr(g["absorption"]), _ptr(g["attenuation"]), m, _ptr(wg["centers"]),
                     _ptr(wall._E), _ptr(wall._ff), int(wall._ff.shape[1]), int(col0), float(speed_of_sound),
                     float(E_sampling_rate), _ptr(ws), wsz, _ptr(err), _stream())
        _raise_for(err, "calculate_energy_exchange")

    def _receiver_device(self, max_order, receiver, speed_of_sound, sampling_rate, out):
        nb, n_orders, n, nt = self._E.shape
        if n == 0:
            return
        g = self._geometry()
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        rcv = _dev(np.asarray(receiver.position, dtype=float).reshape(3))
        nat.call("sp_kang_receiver", n, _ptr(g["centers"]), _ptr(g["normal"]), nb, n_orders, nt, _ptr(self._E),
                 int(max_order), _ptr(rcv), _ptr(g["attenuation"]), float(speed_of_sound), float(sampling_rate),
                 _ptr(out), _ptr(err), _stream())
        _raise_for(err, "energy_at_receiver")

    def energy_at_receiver(self, max_order, receiver, speed_of_sound, sampling_rate):
        """This wall's energy at the receiver, orders 0 .. max_order (RadiosityKang.py:443-498)."""
        out = torch.zeros((self.n_bins, self._E.shape[-1]), dtype=torch.float64, device="cuda")
        self._receiver_device(max_order, receiver, speed_of_sound, sampling_rate, out)
        return out.cpu().numpy()

    # ------------------------------------------------------------ read/write
    def to_dict(self):
        """RadiosityKang.py:107-121."""
        return {'pts': self.pts, 'up_vector': self.up_vector, 'normal': self.normal, 'max_size': self.max_size,
                'other_wall_ids': self.other_wall_ids, 'wall_id': self.wall_id, 'scattering': self.scattering,
                'absorption': self.absorption, 'sound_attenuation_factor': self.sound_attenuation_factor,
                'E_matrix': self.E_matrix}

    @classmethod
    def from_dict(cls, d):
        """RadiosityKang.py:123-133."""
        return cls(Polygon(d['pts'], d['up_vector'], d['normal']), d['max_size'], d['other_wall_ids'], d['wall_id'],
                   d['scattering'], d['absorption'], d['sound_attenuation_factor'], E_matrix=d['E_matrix'])


class RadiosityKang:
    """Kang radiosity over walls (RadiosityKang.py:917-1056)."""

    def __init__(self, walls, patch_size, max_order_k, ir_length_s, speed_of_sound=346.18, sampling_rate=1000,
                 absorption=0.1, source=None):
        self.speed_of_sound = speed_of_sound
        self.max_order_k = max_order_k
        self.sampling_rate = sampling_rate
        self.patch_size = patch_size
        self.ir_length_s = ir_length_s
        n = len(walls)
        self.patch_list = [w if isinstance(w, PatchesKang) else
                           PatchesKang(w, patch_size, [j for j in range(n) if j != i], i, absorption=absorption)
                           for i, w in enumerate(walls)]
        if source is not None:
            self.source = source

    def run(self, source):
        """Source energy, form factors and every exchange order (RadiosityKang.py:1005-1026)."""
        self.source = source
        for p in self.patch_list:
            p.init_energy_exchange(self.max_order_k, self.ir_length_s, source, sampling_rate=self.sampling_rate,
                                   speed_of_sound=self.speed_of_sound)
        if len(self.patch_list) > 1:
            for p in self.patch_list:
                p.calculate_form_factor(self.patch_list)
            for k in range(1, self.max_order_k + 1):
                for p in self.patch_list:
                    p.calculate_energy_exchange(self.patch_list, k, speed_of_sound=self.speed_of_sound,
                                                E_sampling_rate=self.sampling_rate)

    def energy_at_receiver(self, receiver, max_order_k=None, ignore_direct=False):
        """Energy response at the receiver (RadiosityKang.py:1028-1046)."""
        if max_order_k is None:
            max_order_k = self.max_order_k
        m = self.patch_list[0].sound_attenuation_factor
        nb = self.patch_list[0].n_bins
        out = torch.zeros((nb, self.patch_list[0]._E.shape[-1]), dtype=torch.float64, device="cuda")
        for p in self.patch_list:  # each wall's response is added to out in order, as `ir += ...`
            p._receiver_device(max_order_k, receiver, self.speed_of_sound, self.sampling_rate, out)
        ir = out.cpu().numpy()
        if not ignore_direct:
            r = np.sqrt(np.sum((np.asarray(receiver.position) - np.asarray(self.source.position)) ** 2))
            direct_sound = (1 / (4 * np.pi * np.square(r))) * np.exp(-m * r)
            ir[:, int(r / self.speed_of_sound * self.sampling_rate)] += direct_sound
        return ir

    def to_dict(self):
        """RadiosityKang.py:972-986."""
        has = hasattr(self, 'source')
        return {'patch_size': self.patch_size, 'max_order_k': self.max_order_k, 'ir_length_s': self.ir_length_s,
                'speed_of_sound': self.speed_of_sound, 'sampling_rate': self.sampling_rate,
                'patches': [p.to_dict() for p in self.patch_list],
                'source_position': self.source.position if has else None,
                'source_view': self.source.view if has else None, 'source_up': self.source.up if has else None}

    @classmethod
    def from_dict(cls, d):
        """RadiosityKang.py:988-1003."""
        patches = [PatchesKang.from_dict(p) for p in d['patches']]
        source = None
        if d.get('source_position') is not None:
            source = SoundSource(d['source_position'], d['source_view'], d['source_up'])
        return cls(patches, d['patch_size'], d['max_order_k'], d['ir_length_s'], d['speed_of_sound'],
                   d['sampling_rate'], source=source)

    def write(self, filename, compress=True):
        """Write the object to a .far state file (RadiosityKang.py:1048-1051); walls as patch<i>_<key> members."""
        _write_state(self, filename, compress)

    @classmethod
    def from_read(cls, filename):
        """Read an object written by write (RadiosityKang.py:1053-1056)."""
        return cls.from_dict(_read_state(filename, _PATCH_KEYS))


_PATCH_KEYS = ('pts', 'up_vector', 'normal', 'max_size', 'other_wall_ids', 'wall_id', 'scattering', 'absorption',
               'sound_attenuation_factor', 'E_matrix')
_DIRECTIONAL_KEYS = _PATCH_KEYS + ('directivity_data', 'directivity_data_frequencies', 'directivity_sources',
                                   'directivity_receivers', 'directivity_sources_weights',
                                   'directivity_receivers_weights')


def _write_state(obj, filename, compress):
    d = obj.to_dict()
    flat = {k: v for k, v in d.items() if k != 'patches'}
    flat['n_patch_walls'] = len(d['patches'])
    for i, p in enumerate(d['patches']):
        for k, v in p.items():
            flat[f'patch{i}_{k}'] = np.asarray(v) if isinstance(v, np.ndarray) or k in ('pts', 'up_vector',
                                                                                      'normal') else v
    for k in ('source_position', 'source_view', 'source_up'):
        if flat[k] is not None:
            flat[k] = np.asarray(flat[k], dtype=float)
    far.write(filename, flat, compress=compress)


def _none(x):
    return None if isinstance(x, str) and x == 'None' else x


def _read_state(filename, keys):
    v = far.read(filename)
    if 'patches' in v and 'n_patch_walls' not in v:
        # the reference's layout: pyfar.io.write(**to_dict()), the walls as a list of dicts
        d = {k: _none(x) for k, x in v.items() if k != 'patches'}
        d['patches'] = [{k: _none(x) for k, x in p.items()} for p in v['patches']]
        return d
    patches = []
    for i in range(int(v['n_patch_walls'])):
        p = {k: v.get(f'patch{i}_{k}') for k in keys}
        for k in ('E_matrix', 'directivity_sources_weights', 'directivity_receivers_weights'):
            if isinstance(p.get(k), str) and p[k] == 'None':
                p[k] = None
        patches.append(p)
    d = {k: v.get(k) for k in ('patch_size', 'max_order_k', 'ir_length_s', 'speed_of_sound', 'sampling_rate')}
    d['patches'] = patches
    for k in ('source_position', 'source_view', 'source_up'):
        d[k] = None if isinstance(v.get(k), str) else v.get(k)
    return d


# ---------------------------------------------------------------- directional variant
def _orientation(view, up):
    """pyfar's Orientations.from_view_up: the rotation whose matrix rows are view, up and view x up."""
    from scipy.spatial.transform import Rotation
    view = np.atleast_2d(np.asarray(view, dtype=float))
    up = np.atleast_2d(np.asarray(up, dtype=float))
    view = view / np.linalg.norm(view, axis=1)[:, None]
    up = up / np.linalg.norm(up, axis=1)[:, None]
    m = np.empty((view.shape[0], 3, 3))
    m[:, 0], m[:, 1], m[:, 2] = view, up, np.cross(view, up)
    return Rotation.from_matrix(m)


def _rotate_to_wall(xyz, normal, up_vector):
    """RadiosityKang.py:558-567: rotate directions from the data frame (normal +z, up +x) into the wall's
    frame by Euler angles, as pyfar's Coordinates.rotate('xyz', euler) does, then set the radius to 1."""
    from scipy.spatial.transform import Rotation
    o_diff = _orientation(normal, up_vector).inv() * _orientation([0, 0, 1], [1, 0, 0])
    with warnings.catch_warnings():  # axis-aligned walls are gimbal-locked; scipy then sets the third angle to 0
        warnings.simplefilter("ignore", UserWarning)
        euler = o_diff.as_euler('xyz', True).flatten()
    pts = Rotation.from_euler('xyz', euler, degrees=True).apply(np.asarray(xyz, dtype=float).reshape(-1, 3))
    return unit_radius(pts)


def _nearest(points, queries):
    """Index of the nearest point for every query (pyfar's find_nearest: a k-d tree, Euclidean)."""
    from scipy.spatial import cKDTree
    q = np.asarray(queries, dtype=float).reshape(-1, 3)
    if q.shape[0] == 0:
        return np.zeros(0, dtype=np.int32)
    return cKDTree(np.asarray(points, dtype=float).reshape(-1, 3)).query(q)[1].astype(np.int32)


def _coords_copy(c):
    xyz = np.asarray(c.cartesian, dtype=float).reshape(-1, 3)
    w = getattr(c, 'weights', None)
    return Coordinates.from_cartesian(xyz, weights=None if w is None else np.asarray(w, dtype=float).reshape(-1))


class PatchesDirectionalKang(PatchesKang):
    """A wall with directional scattering data (RadiosityKang.py:500-810).

    directivity_data (n_src_dirs, n_dirs, n_bins) over directivity_sources
    (incoming directions) and directivity_receivers (outgoing directions),
    in the wall's frame.  E_matrix is (n_bins, max_order + 1, n_patches,
    n_samples, n_dirs), as the reference's.
    """

    def __init__(self, polygon, max_size, other_wall_ids, wall_id, data, sources, receivers, absorption=None,
                 sound_attenuation_factor=None, already_converted=False, E_matrix=None):
        self.directivity_data = FrequencyData(np.array(data.freq), np.array(data.frequencies))
        if absorption is None:
            absorption = np.zeros_like(self.directivity_data.frequencies) + 0.1
        if sound_attenuation_factor is None:
            sound_attenuation_factor = np.zeros_like(self.directivity_data.frequencies)
        PatchesKang.__init__(self, polygon, max_size, other_wall_ids, wall_id,
                             scattering=np.ones_like(self.directivity_data.frequencies), absorption=absorption,
                             sound_attenuation_factor=sound_attenuation_factor, E_matrix=E_matrix)
        self.directivity_data.freq = np.abs(self.directivity_data.freq)
        self.directivity_sources = _coords_copy(sources)
        self.directivity_receivers = _coords_copy(receivers)
        if not already_converted:
            self.directivity_data.freq = self.directivity_data.freq * np.pi
            for c in (self.directivity_receivers, self.directivity_sources):
                c._pts = _rotate_to_wall(c.cartesian, polygon.normal, polygon.up_vector)

    @classmethod
    def from_sofa(cls, polygon, max_size, other_wall_ids, wall_id, wall_directivity_path, absorption=None,
                  sound_attenuation_factor=None):
        """A wall with the directional data of a SOFA file (RadiosityKang.py:569-584)."""
        from .sofa import convert_sofa, read_sofa
        sofa = read_sofa(wall_directivity_path)
        data, sources, receivers = convert_sofa(sofa)
        sources.weights = getattr(sofa, 'SourceWeights', None)
        receivers.weights = getattr(sofa, 'ReceiverWeights', None)
        assert sources.weights is not None, "No source weights in sofa file"
        assert receivers.weights is not None, "No receiver weights in sofa file"
        return cls(polygon, max_size, other_wall_ids, wall_id, data, sources, receivers, absorption=absorption,
                   sound_attenuation_factor=sound_attenuation_factor)

    # ------------------------------------------------------------ device data
    @property
    def n_dirs(self):
        return int(self.directivity_receivers.csize)

    @property
    def E_matrix(self):
        """(n_bins, max_order + 1, n_patches, n_samples, n_dirs); the device holds it direction-major."""
        return None if self._E is None else np.ascontiguousarray(self._E.cpu().numpy().transpose(0, 1, 2, 4, 3))

    @E_matrix.setter
    def E_matrix(self, value):
        if value is None:
            self._E = None
            return
        value = np.asarray(value, dtype=np.float64)
        if value.ndim != 5:
            raise ValueError("a directional E_matrix is (n_bins, orders, n_patches, n_samples, n_dirs)")
        self._E = _dev(value.transpose(0, 1, 2, 4, 3))
        self.E_n_samples = int(value.shape[3])

    def _table(self):
        freq = np.asarray(self.directivity_data.freq)
        if freq.ndim != 3 or freq.shape[1] != self.n_dirs or freq.shape[2] != self.n_bins:
            raise ValueError(f"directivity data {freq.shape} is not (n_src_dirs, {self.n_dirs}, {self.n_bins})")
        return _dev(np.real(freq))

    def _centers(self):
        return np.sum(self._pts, axis=1) / self._pts.shape[1]

    # ---------------------------------------------------------------- steps
    def init_energy_exchange(self, max_order_k, ir_length_s, source, sampling_rate, speed_of_sound):
        """Source energy per patch and outgoing direction (RadiosityKang.py:629-671)."""
        self.E_sampling_rate = sampling_rate
        self.E_n_samples = int(ir_length_s * sampling_rate)
        n, nd = len(self.patches), self.n_dirs
        nrm = np.abs(np.asarray(self.normal, dtype=float))
        if not (nrm[2] > 0.99 or nrm[1] > 0.99 or nrm[0] > 0.99):
            raise AssertionError()
        self._E = torch.zeros((self.n_bins, max_order_k + 1, n, nd, self.E_n_samples), dtype=torch.float64,
                              device="cuda")
        if n == 0 or self.E_n_samples == 0:
            return
        g = self._geometry()
        idx = _nearest(self.directivity_sources.cartesian,
                       np.asarray(source.position, dtype=float)[None, :] - self._centers())
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        src = _dev(np.asarray(source.position, dtype=float).reshape(3))
        table = self._table()
        idx_d = torch.as_tensor(idx, device="cuda")
        nat.call("sp_kang_directional_init_energy", n, _ptr(g["centers"]), _ptr(g["sizes"]), _ptr(g["normal"]),
                 _ptr(src), float(source.sound_power), self.n_bins, _ptr(g["absorption"]), _ptr(g["attenuation"]),
                 float(speed_of_sound), float(sampling_rate), max_order_k + 1, self.E_n_samples, nd, _ptr(table),
                 _ptr(idx_d), _ptr(self._E), _ptr(err), _stream())
        _raise_for(err, "init_energy_exchange")

    def calculate_energy_exchange(self, patches_list, current_order_k, speed_of_sound, E_sampling_rate):
        """Order k per outgoing direction from the other walls' order k - 1 (RadiosityKang.py:673-745)."""
        k = current_order_k
        n, nd = len(self.patches), self.n_dirs
        nb, n_orders, _, _, nt = self._E.shape
        g = self._geometry()
        table = self._table()
        mine = self._centers()
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        for wid in self.other_wall_ids:
            wall = patches_list[wid]
            if not isinstance(wall, PatchesDirectionalKang) or wall.n_dirs != nd:
                raise ValueError(f"wall {wid} must be directional with {nd} outgoing directions, as this wall")
            m = len(wall.patches)
            if n == 0 or m == 0:
                continue
            # the incoming direction of each (receiver patch, source patch): source centre - receiver centre
            idx = _nearest(self.directivity_sources.cartesian, wall._centers()[None, :, :] - mine[:, None, :])
            idx_d = torch.as_tensor(idx, device="cuda")
            col0 = wall._column(patches_list, self.wall_id)
            wsz = nat.size("sp_kang_exchange_workspace", n, m, nb)
            ws = torch.empty((wsz,), dtype=torch.uint8, device="cuda")
            wg = wall._geometry()
            nat.call("sp_kang_directional_exchange", k, nb, n_orders, nt, n, _ptr(g["centers"]), _ptr(self._E),
                     _ptr(g["scattering"]), _ptr(g["absorption"]), _ptr(g["attenuation"]), m, _ptr(wg["centers"]),
                     _ptr(wall._E), _ptr(wall._ff), int(wall._ff.shape[1]), int(col0), float(speed_of_sound),
                     float(E_sampling_rate), nd, _ptr(table), _ptr(idx_d), _ptr(ws), wsz, _ptr(err), _stream())
        _raise_for(err, "calculate_energy_exchange")

    def _receiver_device(self, max_order, receiver, speed_of_sound, sampling_rate, out):
        nb, n_orders, n, nd, nt = self._E.shape
        if n == 0:
            return
        g = self._geometry()
        # the outgoing direction towards the receiver, moved to radius 1 as the reference does
        dirs = unit_radius(np.asarray(receiver.position, dtype=float)[None, :] - self._centers())
        idx_d = torch.as_tensor(_nearest(self.directivity_receivers.cartesian, dirs), device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        rcv = _dev(np.asarray(receiver.position, dtype=float).reshape(3))
        nat.call("sp_kang_directional_receiver", n, _ptr(g["centers"]), _ptr(g["normal"]), nb, n_orders, nt,
                 _ptr(self._E), int(max_order), _ptr(rcv), _ptr(g["attenuation"]), float(speed_of_sound),
                 float(sampling_rate), nd, _ptr(idx_d), _ptr(out), _ptr(err), _stream())
        _raise_for(err, "energy_at_receiver")

    def energy_at_receiver(self, max_order, receiver, speed_of_sound, sampling_rate):
        """This wall's energy at the receiver, orders 0 .. max_order (RadiosityKang.py:747-810)."""
        out = torch.zeros((self.n_bins, self._E.shape[-1]), dtype=torch.float64, device="cuda")
        self._receiver_device(max_order, receiver, speed_of_sound, sampling_rate, out)
        return out.cpu().numpy()

    # ------------------------------------------------------------ read/write
    def to_dict(self):
        """RadiosityKang.py:586-597."""
        return {**PatchesKang.to_dict(self),
                'directivity_data': self.directivity_data.freq,
                'directivity_data_frequencies': self.directivity_data.frequencies,
                'directivity_sources': self.directivity_sources.cartesian,
                'directivity_receivers': self.directivity_receivers.cartesian,
                'directivity_sources_weights': self.directivity_sources.weights,
                'directivity_receivers_weights': self.directivity_receivers.weights}

    @classmethod
    def from_dict(cls, d):
        """RadiosityKang.py:599-627 (the stored directions are already in the wall's frame)."""
        data = FrequencyData(d['directivity_data'], d['directivity_data_frequencies'])
        src = np.asarray(d['directivity_sources'], dtype=float)
        rcv = np.asarray(d['directivity_receivers'], dtype=float)
        sources = Coordinates(src.T[0], src.T[1], src.T[2], weights=d['directivity_sources_weights'])
        receivers = Coordinates(rcv.T[0], rcv.T[1], rcv.T[2], weights=d['directivity_receivers_weights'])
        return cls(Polygon(d['pts'], d['up_vector'], d['normal']), max_size=d['max_size'],
                   other_wall_ids=d['other_wall_ids'], wall_id=d['wall_id'], data=data, sources=sources,
                   receivers=receivers, absorption=d['absorption'],
                   sound_attenuation_factor=d['sound_attenuation_factor'], E_matrix=d['E_matrix'],
                   already_converted=True)


class DirectionalRadiosityKang:
    """Kang radiosity with directional scattering data per wall (RadiosityKang.py:1059-1202)."""

    def __init__(self, polygon_list, patch_size, max_order_k, ir_length_s, sofa_path, speed_of_sound=346.18,
                 sampling_rate=1000, source=None):
        self.speed_of_sound = speed_of_sound
        self.max_order_k = max_order_k
        self.sampling_rate = sampling_rate
        self.patch_size = patch_size
        self.ir_length_s = ir_length_s
        n = len(polygon_list)
        patch_list = []
        for i in range(n):
            path = sofa_path[i] if isinstance(sofa_path, list) else sofa_path
            w = polygon_list[i]
            patch_list.append(w if isinstance(w, PatchesDirectionalKang) else PatchesDirectionalKang.from_sofa(
                w, self.patch_size, [j for j in range(n) if j != i], i, path))
        self.patch_list = patch_list
        nb = self.patch_list[0].n_bins
        for p in self.patch_list:
            assert p.n_bins == nb, f'Number of bins is not the same for all patches. {p.n_bins} != {nb}'
        if source is not None:
            self.source = source

    def run(self, source):
        """Source energy, form factors and every exchange order (RadiosityKang.py:1163-1184)."""
        RadiosityKang.run(self, source)

    def energy_at_receiver(self, receiver, order_k=None):
        """Energy response at the receiver, direct sound included (RadiosityKang.py:1186-1202)."""
        return RadiosityKang.energy_at_receiver(self, receiver, max_order_k=order_k)

    def to_dict(self):
        """RadiosityKang.py:1126-1141."""
        return RadiosityKang.to_dict(self)

    @classmethod
    def from_dict(cls, d):
        """RadiosityKang.py:1143-1161."""
        patches = [PatchesDirectionalKang.from_dict(p) for p in d['patches']]
        source = None
        if d.get('source_position') is not None:
            source = SoundSource(d['source_position'], d['source_view'], d['source_up'])
        return cls(patches, d['patch_size'], d['max_order_k'], d['ir_length_s'], sofa_path=None,
                   speed_of_sound=d['speed_of_sound'], sampling_rate=d['sampling_rate'], source=source)

    def write(self, filename, compress=True):
        """Write the object to a .far state file (RadiosityKang.py:1116-1118)."""
        _write_state(self, filename, compress)

    @classmethod
    def from_read(cls, filename):
        """Read an object written by write (RadiosityKang.py:1120-1124)."""
        return cls.from_dict(_read_state(filename, _DIRECTIONAL_KEYS))
