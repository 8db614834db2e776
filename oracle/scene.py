"""Scene arrays for the oracle, taken from a configured radiosity object.

TEST INFRASTRUCTURE: converts the host-side inputs of a
sparrowpy_gb300.DirectionalRadiosityFast (patches, walls, rotated BRDF
direction sets, BRDF tables already times pi, BRDF index, air attenuation)
into the plain-array scene the oracle consumes.  Both sides therefore
receive identical inputs.
"""
import numpy as np


def scene_from_radiosity(r):
    has_brdf = r._brdf_incoming_directions is not None
    sc = dict(
        patches_points=np.asarray(r._patches_points, float),
        patch_to_wall_ids=np.asarray(r._patch_to_wall_ids, np.int64),
        walls_points=np.asarray(r._walls_points, float),
        walls_normal=np.asarray(r._walls_normal, float),
        air_attenuation=None if r._air_attenuation is None else np.asarray(r._air_attenuation, float),
    )
    if has_brdf:
        sc["dirs_in"] = np.array([np.asarray(c.cartesian, float).reshape(-1, 3) for c in r._brdf_incoming_directions])
        sc["dirs_out"] = np.array([np.asarray(c.cartesian, float).reshape(-1, 3) for c in r._brdf_outgoing_directions])
        slots = []
        for b in r._brdf:
            b = np.asarray(b, float)
            slots.append(b.reshape(1, 1, -1) if b.ndim == 1 else b)
        sc["brdf"] = np.array(slots)
        sc["brdf_index"] = np.asarray(r._brdf_index, np.int64)
    else:
        sc["dirs_in"] = None
        sc["dirs_out"] = None
    return sc
