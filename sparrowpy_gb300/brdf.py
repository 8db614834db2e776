"""Direction samplings and BRDF construction (host-side inputs).

`create_from_scattering` and `create_from_directional_scattering` restate
sparrowpy/brdf.py:8-225 and return the tables; writing them to a SOFA file
(`file_path`) is not provided and raises NotImplementedError.  `sph_gaussian` restates the Gauss-Legendre sphere sampling
the reference tests draw their BRDF directions from (pyfar.samplings).
"""
import numpy as np

from .coords import Coordinates, FrequencyData, _cart, is_frequency_data


def sph_gaussian(n_points=None, sh_order=None, radius=1.0):
    """Gauss-Legendre sampling: n_theta colatitude nodes x n_phi azimuths.

    ``sh_order`` gives n_points = (sh_order + 1, 2 (sh_order + 1)).  Points
    are ordered azimuth-major; weights sum to 1.
    """
    if n_points is None:
        if sh_order is None:
            raise ValueError("give n_points or sh_order")
        n_points = (sh_order + 1, 2 * (sh_order + 1))
    n_points = np.atleast_1d(n_points)
    if n_points.size == 1:
        n_points = np.array([n_points[0], n_points[0]])
    n_theta, n_phi = int(n_points[0]), int(n_points[1])
    legendre, weights = np.polynomial.legendre.leggauss(n_theta)
    theta_angles = np.arccos(legendre)
    phi_angles = np.arange(0, 2 * np.pi, 2 * np.pi / n_phi)
    theta, phi = np.meshgrid(theta_angles, phi_angles)
    w = np.tile(weights, n_phi)
    w = w / np.sum(w)
    return Coordinates.from_spherical_colatitude(phi.reshape(-1), theta.reshape(-1), radius, weights=w)


def hemisphere_directions(n_directions):
    """Upper-hemisphere (z > 0) Gauss-Legendre directions with weights.

    Supported counts: 1 (the normal), 4, 8, 16, 32, 64, 128 (mirror-closed:
    the azimuth + pi image of every direction is in the set).
    """
    table = {4: (2, 4), 8: (2, 8), 16: (4, 8), 32: (8, 8), 64: (8, 16), 128: (16, 16)}
    if n_directions == 1:
        return Coordinates(0.0, 0.0, 1.0, weights=1.0)
    if n_directions not in table:
        raise ValueError(f"unsupported number of directions {n_directions}")
    g = sph_gaussian(n_points=table[n_directions])
    keep = g.z > 0
    out = Coordinates.from_cartesian(g.cartesian[keep], weights=g.weights[keep])
    assert out.csize == n_directions
    return out


def _no_sofa_output(file_path):
    if file_path is not None:
        raise NotImplementedError("writing SOFA files is not provided; the BRDF is returned as FrequencyData")


def create_from_scattering(source_directions, receiver_directions, scattering_coefficient,
                           absorption_coefficient=None, file_path=None):
    """Diffuse-plus-mirror BRDF (sparrowpy/brdf.py:8-130).

    rho(i, o) = s(1-a)/pi + (1-s)(1-a)/(cos(theta) w) [o == mirror(i)],
    returned as FrequencyData of shape (n_sources, n_receivers, n_bins).
    The cosine/weight factor is indexed exactly as in brdf.py:110-118.
    """
    if not is_frequency_data(scattering_coefficient) or tuple(scattering_coefficient.cshape) != (1,):
        raise TypeError('scattering_coefficient must be a pf.FrequencyData object with shape (1,)')
    if not hasattr(source_directions, "cartesian"):
        raise TypeError('source_directions must be a pf.Coordinates object')
    if not hasattr(receiver_directions, "cartesian"):
        raise TypeError('receiver_directions must be a pf.Coordinates object')
    _no_sofa_output(file_path)
    freqs = np.asarray(scattering_coefficient.frequencies)
    if absorption_coefficient is None:
        absorption_coefficient = FrequencyData(np.zeros_like(freqs), freqs)
    src = _cart(source_directions).reshape(-1, 3)
    rcv = _cart(receiver_directions).reshape(-1, 3)
    n_bins = freqs.size
    brdf = np.zeros((src.shape[0], rcv.shape[0], n_bins))
    w = np.asarray(receiver_directions.weights, dtype=float).reshape(-1).copy()
    w *= 2 * np.pi / np.sum(w)
    s = np.real(np.asarray(scattering_coefficient.freq).flatten())
    # image source: azimuth + pi (same colatitude)
    r = np.sqrt(np.sum(src ** 2, axis=-1))
    colat = np.arccos(np.clip(src[:, 2] / r, -1, 1))
    az = np.arctan2(src[:, 1], src[:, 0]) + np.pi
    image = np.stack([r * np.sin(colat) * np.cos(az), r * np.sin(colat) * np.sin(az), r * np.cos(colat)], axis=-1)
    d = np.sum((rcv[None, :, :] - image[:, None, :]) ** 2, axis=-1)
    i_receiver = np.argmin(d, axis=1)
    cos_factor = np.cos(colat[np.newaxis, ...]) * w[..., np.newaxis]
    scattering_factor = 1 - s[np.newaxis, ...]
    brdf[:, :, :] += s / np.pi
    i_sources = np.arange(src.shape[0])
    brdf[i_sources, i_receiver, :] += scattering_factor / cos_factor[i_sources, i_receiver, np.newaxis]
    brdf *= (1 - np.asarray(absorption_coefficient.freq).flatten())
    return FrequencyData(brdf, freqs)


def create_from_directional_scattering(source_directions, receiver_directions, directional_scattering,
                                       absorption_coefficient=None, file_path=None):
    """BRDF from a directional scattering coefficient s_d (sparrowpy/brdf.py:133-225).

    rho(i, o) = (1 - a) s_d(i, o) / (cos(theta_o) w_o), with the receiver
    weights scaled to sum to 2 pi; directional_scattering is FrequencyData
    of cshape (n_sources, n_receivers).  Returned as FrequencyData
    (n_sources, n_receivers, n_bins) at the absorption's frequencies.
    """
    if not hasattr(source_directions, "cartesian"):
        raise TypeError('source_directions must be a pf.Coordinates object')
    if not hasattr(receiver_directions, "cartesian"):
        raise TypeError('receiver_directions must be a pf.Coordinates object')
    n_src = int(np.prod(np.shape(_cart(source_directions))[:-1]))
    n_rcv = int(np.prod(np.shape(_cart(receiver_directions))[:-1]))
    if not is_frequency_data(directional_scattering) or \
            tuple(np.shape(directional_scattering.freq)[:-1]) != (n_src, n_rcv):
        raise TypeError('directional_scattering must be a pf.FrequencyData object with'
                        f' cshape ({n_src, n_rcv})')
    _no_sofa_output(file_path)
    freqs = np.asarray(directional_scattering.frequencies)
    if absorption_coefficient is None:
        absorption_coefficient = FrequencyData(np.zeros_like(freqs), freqs)
    rcv = _cart(receiver_directions).reshape(-1, 3)
    colat = np.arccos(np.clip(rcv[:, 2] / np.sqrt(np.sum(rcv ** 2, axis=-1)), -1, 1))
    cos_receiver = np.cos(colat)[np.newaxis, :, np.newaxis]
    w = np.asarray(receiver_directions.weights, dtype=float).reshape(-1).copy()
    w *= 2 * np.pi / np.sum(w)
    brdf = np.asarray(directional_scattering.freq) / w[..., np.newaxis] / cos_receiver
    brdf = brdf * (1 - np.asarray(absorption_coefficient.freq).flatten())
    return FrequencyData(brdf, np.asarray(absorption_coefficient.frequencies))
