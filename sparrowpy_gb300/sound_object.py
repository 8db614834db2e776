"""Sound sources and receivers with position, orientation and directivity (sparrowpy/sound_object.py:8-218).

init_source_energy takes a SoundSource as well as a Coordinates point; with a
directivity, the source energy of every patch and band is multiplied by the
directivity value towards the patch centre (RadiosityFast.py:500-519).

DirectivityMS holds a directivity as data (n_points, n_frequencies) over
sampled directions (Coordinates) in the source's frame. As in the
reference it is read from a SOFA file (FreeFieldDirectivityTF): the
emitter `source_index` of Data_Real + 1j Data_Imag at the frequencies N,
over the receiver positions (sofa.py reads the file without sofar).
DirectivityMS.from_arrays builds one from data.
"""
import numpy as np

from .coords import Coordinates, FrequencyData, _cart


def _get_metrics(pos_G, view_G, up_G, target_pos_G):
    """Azimuth and elevation (degrees) of target_pos_G seen from a source at pos_G (sound_object.py:77-96).

    The source frame has x' = view x up, y' = up and z' = -view.  The azimuth
    is atan2(-w_x', -w_z') and the elevation asin(w_y' / |w|) of the target
    direction w.  The convention is the reference's, so that directivity
    data sampled for it reads the same.  target_pos_G may be (3,) or (n, 3).
    """
    pos = np.asarray(pos_G, dtype=float)
    view = np.asarray(view_G, dtype=float)
    up = np.asarray(up_G, dtype=float)
    w_g = np.asarray(target_pos_G, dtype=float) - pos
    x_dash = np.cross(view, up)
    w = np.stack([w_g @ x_dash, w_g @ up, w_g @ (-view)], axis=-1)
    azimuth_deg = np.arctan2(-w[..., 0], -w[..., 2]) / np.pi * 180
    elevation_deg = np.arcsin(w[..., 1] / np.sqrt(np.sum(w * w, axis=-1))) / np.pi * 180
    return azimuth_deg, elevation_deg


class DirectivityMS:
    """Directivity of a source: complex data (n_points, n_frequencies) over sampled directions."""

    def __init__(self, file_path=None, source_index=0, *, data=None, receivers=None):
        if file_path is not None:
            # sound_object.py:26-40
            from .sofa import read_sofa, sofa_pos
            sofa = read_sofa(file_path)
            data = FrequencyData(np.asarray(sofa.Data_Real)[source_index, :] +
                                 1j * np.asarray(sofa.Data_Imag)[source_index, :], sofa.N)
            positions = np.asarray(sofa.ReceiverPosition)
            if positions.ndim > 2:
                positions = np.squeeze(positions)
            receivers = sofa_pos(sofa.ReceiverPosition_Type, positions)
            if receivers.cdim != 1:
                raise ValueError("DirectivityMS only supports 1D coordinates, "
                                 f"got {receivers.cdim}D coordinates. Squeezing did not work.")
        if data is None or receivers is None:
            raise ValueError("a directivity needs data (FrequencyData) and receivers (Coordinates)")
        if np.asarray(data.freq).shape[0] != receivers.csize:
            raise ValueError("one row of directivity data per receiver direction")
        self.data = data
        self.receivers = receivers

    @classmethod
    def from_arrays(cls, data, frequencies, directions):
        """data (n_points, n_frequencies) complex or real, frequencies (n,), directions (n_points, 3) or Coordinates."""
        receivers = directions if isinstance(directions, Coordinates) else \
            Coordinates.from_cartesian(np.asarray(directions, dtype=float).reshape(-1, 3))
        return cls(data=FrequencyData(np.asarray(data), frequencies), receivers=receivers)

    def get_directivity(self, source_pos, source_view, source_up, target_position, i_freq):
        """Directivity value of the sampled direction nearest to the target (sound_object.py:42-73)."""
        az, el = _get_metrics(source_pos, source_view, source_up, target_position)
        find = Coordinates.from_spherical_elevation(np.atleast_1d(az) / 180 * np.pi,
                                                    np.atleast_1d(el) / 180 * np.pi, 1)
        index, _ = self.receivers.find_nearest(find)
        return np.asarray(self.data.freq)[index[0], i_freq]


class SoundObject:
    """Position, view and up vector of a source or receiver (sound_object.py:99-126)."""

    def __init__(self, position, view, up):
        self.position = np.array(position, dtype=float)
        assert self.position.shape == (3,)
        self.view = np.array(view, dtype=float)
        assert self.view.shape == (3,)
        self.view /= np.sqrt(np.dot(self.view, self.view))
        self.up = np.array(up, dtype=float)
        assert self.up.shape == (3,)
        self.up /= np.sqrt(np.dot(self.up, self.up))


class SoundSource(SoundObject):
    """A source with an optional directivity and a sound power in W (sound_object.py:142-206)."""

    def __init__(self, position, view, up, directivity=None, sound_power=1):
        super().__init__(position, view, up)
        self.sound_power = float(sound_power)
        if directivity is not None:
            assert isinstance(directivity, DirectivityMS)
        self.directivity = directivity

    def get_directivity(self, target_position, frequency):
        """Directivity towards target_position ((3,) or (n, 3)) at the frequency bin nearest to frequency."""
        i_freq = int(np.argmin(np.abs(np.asarray(self.directivity.data.frequencies) - frequency)))
        target = np.asarray(target_position, dtype=float)
        return self.directivity.get_directivity(self.position, self.view, self.up, target.reshape(-1, 3), i_freq)


class Receiver(SoundObject):
    """A receiver with position and orientation (sound_object.py:208-218)."""


def directions(coords):
    """Cartesian (n, 3) of a Coordinates object (helper for building DirectivityMS data)."""
    return _cart(coords).reshape(-1, 3)
