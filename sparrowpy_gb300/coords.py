"""Small stand-ins for the pyfar containers the radiosity API exchanges.

sparrowpy's ``DirectionalRadiosityFast`` takes and returns pyfar objects
(``Coordinates``, ``FrequencyData``, ``TimeData``).  pyfar is not required
here: these classes provide the attributes the radiosity path reads
(``cartesian``, ``weights``, ``cshape``, ``csize``, ``cdim``, ``x/y/z``,
``colatitude``, ``azimuth``, ``radius``, ``copy``, ``find_nearest``;
``freq``, ``frequencies``, ``n_bins``; ``time``, ``times``), and every
function of this package also accepts real pyfar objects by duck typing.
"""
import numpy as np


class Coordinates:
    """Cartesian points with optional sampling weights (pyfar-like)."""

    def __init__(self, x=None, y=None, z=None, weights=None):
        if x is None:
            pts = np.zeros((0, 3))
        else:
            x = np.atleast_1d(np.asarray(x, dtype=float))
            y = np.atleast_1d(np.asarray(y, dtype=float))
            z = np.atleast_1d(np.asarray(z, dtype=float))
            x, y, z = np.broadcast_arrays(x, y, z)
            pts = np.stack([x, y, z], axis=-1)
        self._pts = np.array(pts, dtype=float)
        if weights is not None:
            weights = np.broadcast_to(np.asarray(weights, dtype=float), self._pts.shape[:-1]).copy()
        self._weights = weights

    @classmethod
    def from_cartesian(cls, xyz, weights=None):
        xyz = np.asarray(xyz, dtype=float)
        return cls(xyz[..., 0], xyz[..., 1], xyz[..., 2], weights=weights)

    @classmethod
    def from_spherical_colatitude(cls, azimuth, colatitude, radius=1.0, weights=None):
        azimuth, colatitude, radius = np.broadcast_arrays(
            np.asarray(azimuth, float), np.asarray(colatitude, float), np.asarray(radius, float))
        x = radius * np.sin(colatitude) * np.cos(azimuth)
        y = radius * np.sin(colatitude) * np.sin(azimuth)
        z = radius * np.cos(colatitude)
        return cls(x, y, z, weights=weights)

    @classmethod
    def from_spherical_elevation(cls, azimuth, elevation, radius=1.0, weights=None):
        """Points from azimuth, elevation (radians) and radius, as pyfar computes them (see sph2cart)."""
        x, y, z = sph2cart(azimuth, np.pi / 2 - np.asarray(elevation, float), radius)
        return cls(x, y, z, weights=weights)

    @property
    def cartesian(self):
        return self._pts

    @property
    def x(self):
        return self._pts[..., 0]

    @property
    def y(self):
        return self._pts[..., 1]

    @property
    def z(self):
        return self._pts[..., 2]

    @property
    def weights(self):
        return self._weights

    @weights.setter
    def weights(self, w):
        self._weights = None if w is None else np.broadcast_to(
            np.asarray(w, dtype=float), self.cshape).copy()

    @property
    def cshape(self):
        return self._pts.shape[:-1]

    @property
    def csize(self):
        return int(np.prod(self.cshape))

    @property
    def cdim(self):
        return len(self.cshape)

    @property
    def radius(self):
        return np.sqrt(np.sum(self._pts ** 2, axis=-1))

    @radius.setter
    def radius(self, r):
        cur = self.radius
        self._pts = self._pts / cur[..., None] * np.asarray(r, float)[..., None]

    @property
    def colatitude(self):
        return np.arccos(np.clip(self.z / self.radius, -1.0, 1.0))

    @property
    def azimuth(self):
        return np.mod(np.arctan2(self.y, self.x), 2 * np.pi)

    @azimuth.setter
    def azimuth(self, az):
        r, col = self.radius, self.colatitude
        az = np.asarray(az, dtype=float)
        self._pts = np.stack([r * np.sin(col) * np.cos(az), r * np.sin(col) * np.sin(az), r * np.cos(col)], axis=-1)

    def copy(self):
        c = Coordinates()
        c._pts = self._pts.copy()
        c._weights = None if self._weights is None else self._weights.copy()
        return c

    def __eq__(self, other):
        """Equal points and weights (content, as pyfar compares Coordinates)."""
        if not isinstance(other, Coordinates):
            return NotImplemented
        if self._pts.shape != other._pts.shape or not np.array_equal(self._pts, other._pts):
            return False
        if (self._weights is None) != (other._weights is None):
            return False
        return self._weights is None or np.array_equal(self._weights, other._weights)

    __hash__ = None

    def __getitem__(self, idx):
        c = Coordinates()
        c._pts = np.atleast_2d(self._pts[idx])
        if self._weights is not None:
            c._weights = np.atleast_1d(self._weights[idx])
        return c

    def __sub__(self, other):
        return Coordinates.from_cartesian(self._pts - _cart(other))

    def find_nearest(self, points):
        """Index of the nearest point (Euclidean) for every query point, and its distance.

        As pyfar's find_nearest, a k-d tree (scipy's cKDTree) answers the
        query, so that exact ties resolve the same way.
        """
        from scipy.spatial import cKDTree
        q = _cart(points).reshape(-1, 3)
        if q.shape[0] == 0 or self.csize == 0:
            return (np.zeros(q.shape[0], dtype=int),), np.full(q.shape[0], np.inf)
        dist, idx = cKDTree(self._pts.reshape(-1, 3)).query(q)
        return (np.asarray(idx, dtype=int),), np.asarray(dist)


def sph2cart(azimuth, colatitude, radius):
    """Spherical to cartesian as pyfar's `sph2cart`: x = (r sin col) cos az, y = (r sin col) sin az,
    z = r cos col, with components below the FP64 epsilon in magnitude set to 0."""
    azimuth, colatitude, radius = (np.atleast_1d(np.asarray(v, float)) for v in (azimuth, colatitude, radius))
    r_sin_col = radius * np.sin(colatitude)
    x = r_sin_col * np.cos(azimuth)
    y = r_sin_col * np.sin(azimuth)
    z = radius * np.cos(colatitude)
    eps = np.finfo(float).eps
    for v in (x, y, z):
        v[np.abs(v) < eps] = 0
    return x, y, z


def cart2sph(x, y, z):
    """Cartesian to (azimuth in [0, 2 pi), colatitude, radius) as pyfar's `cart2sph`."""
    radius = np.sqrt(x ** 2 + y ** 2 + z ** 2)
    z_div_r = np.divide(z, radius, out=np.zeros_like(radius, dtype=float), where=radius != 0)
    return np.mod(np.arctan2(y, x), 2 * np.pi), np.arccos(z_div_r), radius


def unit_radius(xyz):
    """Points moved to radius 1 through spherical coordinates, as assigning pyfar's `radius = 1` does."""
    xyz = np.asarray(xyz, float)
    az, col, _ = cart2sph(xyz[..., 0], xyz[..., 1], xyz[..., 2])
    x, y, z = sph2cart(az, col, np.ones_like(az))
    return np.stack([x, y, z], axis=-1).reshape(xyz.shape)


class FrequencyData:
    """Frequency-domain data ``freq`` (..., n_bins) at ``frequencies`` (real or complex, as given)."""

    def __init__(self, data, frequencies):
        data = np.asarray(data)
        self.freq = np.atleast_1d(data.astype(complex if np.iscomplexobj(data) else float))
        self.frequencies = np.atleast_1d(np.asarray(frequencies, dtype=float))
        if self.freq.shape[-1] != self.frequencies.size:
            raise ValueError("last dimension of data must match the number of frequencies")

    @property
    def n_bins(self):
        return self.frequencies.size

    @property
    def cshape(self):
        return self.freq.shape[:-1] if self.freq.ndim > 1 else (1,)


class TimeData:
    """Time-domain data ``time`` (..., n_samples) at ``times``."""

    def __init__(self, data, times):
        self.time = np.asarray(data)
        self.times = np.asarray(times, dtype=float)

    @property
    def cshape(self):
        return self.time.shape[:-1]

    @property
    def n_samples(self):
        return self.time.shape[-1]


def _cart(obj):
    """Cartesian (…, 3) array of a Coordinates-like object or array."""
    if hasattr(obj, "cartesian"):
        return np.asarray(obj.cartesian, dtype=float)
    return np.asarray(obj, dtype=float)


def is_coordinates(obj):
    return hasattr(obj, "cartesian") and hasattr(obj, "cshape")


def is_frequency_data(obj):
    return hasattr(obj, "freq") and hasattr(obj, "frequencies")
