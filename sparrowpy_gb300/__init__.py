"""GB300-native directional fast radiosity (sparrowpy's hot path on sm_103a).

Drop-in for ``sparrowpy.DirectionalRadiosityFast``; see radiosity.py.
"""
from . import brdf, form_factor, geometry, kang, mesh, sofa, sound_object, testing, utils
from .coords import Coordinates, FrequencyData, TimeData
from .geometry import Polygon, shoebox_room_stub
from .kang import DirectionalRadiosityKang, PatchesDirectionalKang, PatchesKang, RadiosityKang
from .radiosity import DirectionalRadiosityFast, analyse_brdf

__version__ = "0.1.0"

__all__ = [
    "DirectionalRadiosityFast", "Polygon", "shoebox_room_stub", "Coordinates", "FrequencyData", "TimeData",
    "brdf", "geometry", "sound_object", "analyse_brdf", "kang", "mesh", "sofa", "PatchesKang", "RadiosityKang",
    "PatchesDirectionalKang", "DirectionalRadiosityKang", "form_factor", "testing", "utils",
]
