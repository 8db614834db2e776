"""SOFA files (AES69) as sparrowpy reads them, without sofar, netCDF4 or pyfar.

sparrowpy reads SOFA files in two places:

* ``DirectivityMS(file_path)`` (sound_object.py:13-40): a source
  directivity of the FreeFieldDirectivityTF convention, through
  ``sofar.read_sofa`` and ``pyfar.io.io._sofa_pos``;
* ``PatchesDirectionalKang.from_sofa`` (classes/RadiosityKang.py:570-584):
  a wall's directional scattering data of the GeneralTF convention,
  through ``sofar.read_sofa`` and ``pyfar.io.convert_sofa``, plus the
  ``SourceWeights`` and ``ReceiverWeights`` variables.

``read_sofa`` reads the file's HDF5 container with ``hdf5.File`` and names
its variables as sofar does: a variable ``Data.Real`` becomes the attribute
``Data_Real``, a variable attribute ``Type`` of ``ReceiverPosition`` becomes
``ReceiverPosition_Type``, and a global attribute ``DataType`` becomes
``GLOBAL_DataType``.  netCDF's bare dimensions (datasets that only carry a
dimension's length) are left out.  ``sofa_pos`` and ``convert_sofa``
restate pyfar's conversion of positions and data.
"""
import numpy as np

from . import hdf5
from .coords import Coordinates, FrequencyData

_NETCDF_DIMENSION = "This is a netCDF dimension but not a netCDF variable"
_INTERNAL_ATTRS = {"DIMENSION_LIST", "REFERENCE_LIST", "CLASS", "NAME", "_Netcdf4Dimid", "_Netcdf4Coordinates",
                   "_nc3_strict", "_NCProperties"}


class SofaFile:
    """The variables and attributes of a SOFA file, named as sofar names them."""

    def __init__(self, path):
        self.path = str(path)
        f = hdf5.File(self.path)
        for name, attr in f.attrs.items():
            if name not in _INTERNAL_ATTRS:
                setattr(self, "GLOBAL_" + name, attr.value())
        self._variables = []
        for name, ds in f.datasets().items():
            nm = ds.attrs.get("NAME")
            if nm is not None and str(nm.value()).startswith(_NETCDF_DIMENSION):
                continue
            key = name.replace(".", "_")
            setattr(self, key, ds.read())
            self._variables.append(key)
            for aname, attr in ds.attrs.items():
                if aname not in _INTERNAL_ATTRS:
                    setattr(self, f"{key}_{aname}", attr.value())

    @property
    def variables(self):
        """Names of the variables read (sofar spelling)."""
        return list(self._variables)


def read_sofa(path):
    """Read a SOFA file (sofar.read_sofa without its convention checks)."""
    return SofaFile(path)


def sofa_pos(pos_type, positions):
    """Positions (n, 3) as Coordinates, as pyfar's `_sofa_pos`: `spherical` rows are (azimuth deg,
    elevation deg, radius), `cartesian` rows (x, y, z)."""
    positions = np.asarray(positions, dtype=float)
    if pos_type == "spherical":
        return Coordinates.from_spherical_elevation(positions[:, 0] / 180 * np.pi, positions[:, 1] / 180 * np.pi,
                                                    positions[:, 2])
    if pos_type == "cartesian":
        return Coordinates(positions[:, 0], positions[:, 1], positions[:, 2])
    raise ValueError(f"Position:Type {pos_type} is not supported.")


def convert_sofa(sofa):
    """(data, sources, receivers) of a transfer-function SOFA file, as pyfar's `convert_sofa` for TF data:
    data = Data_Real + 1j Data_Imag at the frequencies N; positions through `sofa_pos`."""
    dtype = str(getattr(sofa, "GLOBAL_DataType", ""))
    if not dtype.startswith("TF"):
        raise NotImplementedError(f"SOFA DataType '{dtype}': only transfer-function data (TF) is read here")
    data = FrequencyData(np.asarray(sofa.Data_Real) + 1j * np.asarray(sofa.Data_Imag), np.asarray(sofa.N))
    sources = sofa_pos(sofa.SourcePosition_Type, np.asarray(sofa.SourcePosition).reshape(-1, 3))
    receivers = sofa_pos(sofa.ReceiverPosition_Type, np.squeeze(np.asarray(sofa.ReceiverPosition)).reshape(-1, 3))
    return data, sources, receivers
