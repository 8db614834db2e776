"""State files for DirectionalRadiosityFast.write / from_read (RadiosityFast.py:828-839).

A file is a zip archive. Its members follow the layout of the reference's
pyfar `.far` files:

* `<name>/$ndarray`: one numpy `.npy` member per array;
* `builtin_wrapper/$BuiltinsWrapper`: one JSON object holding every other
  value (numbers, strings, nested lists; None is written as 'None', as
  RadiosityFast.to_dict does).

Two kinds of values have no pyfar-independent encoding, and get their own
members:

* per-wall direction sets (Coordinates): `<name>/cartesian/$ndarray`
  (n_walls, n, 3) and `<name>/weights/$ndarray`;
* the list of BRDF tables: `<name>/<i>/$ndarray`, one per slot.

The JSON object names them under "sparrowpy_gb300.encoding".

Files the reference writes (pyfar.io.write of RadiosityFast.to_dict, whose
arrays are nested lists) are read through pyfar's codec, restated: a value
['$<type>', payload] is a type hint, '$ndarray' naming the npy member that
holds the array (as `signal/_data` in the reference's test data files),
'$Coordinates' the object's attribute dict (its cartesian points `_data`
and `_weights`), '$tuple' and '$dtype' and numpy scalar types their
values; a top-level object member is `<name>/$<type>`.  Other pyfar types
are refused with their name.
"""
import io
import json
import zipfile

import numpy as np

from .coords import Coordinates, _cart, is_coordinates

FORMAT = "sparrowpy_gb300.state 1"
_BUILTINS = "builtin_wrapper/$BuiltinsWrapper"


def _npy_bytes(a):
    buf = io.BytesIO()
    np.save(buf, np.ascontiguousarray(a), allow_pickle=False)
    return buf.getvalue()


def _npy_load(b):
    return np.load(io.BytesIO(b), allow_pickle=False)


def write(filename, values, compress=True):
    """Write a dict of arrays, per-wall Coordinates arrays, lists of arrays and builtins."""
    builtins, encoding, members = {"sparrowpy_gb300.format": FORMAT}, {}, {}
    for name, v in values.items():
        if isinstance(v, np.ndarray) and v.dtype == object and v.size and all(is_coordinates(c) for c in v.ravel()):
            cart = np.stack([_cart(c).reshape(-1, 3) for c in v.ravel()])
            w = np.stack([np.asarray(c.weights, dtype=float).reshape(-1) if c.weights is not None
                          else np.full(cart.shape[1], np.nan) for c in v.ravel()])
            members[f"{name}/cartesian/$ndarray"] = _npy_bytes(cart)
            members[f"{name}/weights/$ndarray"] = _npy_bytes(w)
            encoding[name] = "coordinates_per_wall"
        elif isinstance(v, list) and v and all(isinstance(a, np.ndarray) for a in v):
            for i, a in enumerate(v):
                members[f"{name}/{i}/$ndarray"] = _npy_bytes(a)
            encoding[name] = ["ndarray_list", len(v)]
        elif isinstance(v, np.ndarray) and v.dtype != object:
            members[f"{name}/$ndarray"] = _npy_bytes(v)
        else:
            builtins[name] = "None" if v is None else (v.item() if isinstance(v, np.generic) else v)
    builtins["sparrowpy_gb300.encoding"] = encoding
    mode = zipfile.ZIP_DEFLATED if compress else zipfile.ZIP_STORED
    with zipfile.ZipFile(filename, "w", compression=mode) as z:
        for m, b in members.items():
            z.writestr(m, b)
        z.writestr(_BUILTINS, json.dumps(builtins))


def _coordinates_from_pyfar(d):
    """Coordinates from a pyfar Coordinates attribute dict (cartesian `_data`, or `_x`, `_y`, `_z`)."""
    if "_data" in d:
        xyz = np.asarray(d["_data"], dtype=float)
    elif all(k in d for k in ("_x", "_y", "_z")):
        xyz = np.stack([np.asarray(d[k], dtype=float) for k in ("_x", "_y", "_z")], axis=-1)
    else:
        raise NotImplementedError(f"a Coordinates object with members {sorted(d)} cannot be read here")
    w = d.get("_weights")
    w = None if w is None or (isinstance(w, str) and w == "None") else np.asarray(w, dtype=float)
    return Coordinates.from_cartesian(xyz, weights=w)


def _pyfar_decode(obj, z):
    """A value of the pyfar codec with its type hints resolved (arrays loaded from their zip members)."""
    if isinstance(obj, list):
        if len(obj) == 2 and isinstance(obj[0], str) and obj[0].startswith("$"):
            hint, payload = obj[0][1:], obj[1]
            if hint == "ndarray":
                return _npy_load(z.read(payload))
            if hint == "Coordinates":
                return _coordinates_from_pyfar(_pyfar_decode(payload, z))
            if hint == "tuple":
                return tuple(_pyfar_decode(payload, z))
            if hint == "dtype":
                return np.dtype(payload)
            scalar = getattr(np, hint, None)
            if isinstance(scalar, type) and issubclass(scalar, np.generic):
                return scalar(payload)
            raise NotImplementedError(f"pyfar type '{hint}' cannot be read here")
        return [_pyfar_decode(x, z) for x in obj]
    if isinstance(obj, dict):
        return {k: _pyfar_decode(v, z) for k, v in obj.items()}
    return obj


def read(filename):
    """Read a file written by write(), or a pyfar file (the reference's write()) of arrays, builtins and
    Coordinates."""
    values, arrays = {}, {}
    with zipfile.ZipFile(filename, "r") as z:
        for m in z.namelist():
            head, _, last = m.rpartition("/")
            if m == _BUILTINS:
                values.update(_pyfar_decode(json.loads(z.read(m).decode("utf-8")), z))
            elif last == "$ndarray":
                arrays[head] = _npy_load(z.read(m))
            elif last == "$Coordinates" and "/" not in head:
                values[head] = _pyfar_decode(["$Coordinates", json.loads(z.read(m).decode("utf-8"))], z)
            elif last.startswith("$"):
                raise NotImplementedError(f"member '{m}': pyfar type '{last[1:]}' cannot be read here")
            # any other member is the payload of a type hint, read where it is named
    encoding = values.pop("sparrowpy_gb300.encoding", {})
    values.pop("sparrowpy_gb300.format", None)
    values.pop("pyfar.__version__", None)
    for name, kind in encoding.items():
        if kind == "coordinates_per_wall":
            cart, w = arrays.pop(f"{name}/cartesian"), arrays.pop(f"{name}/weights")
            out = np.empty(cart.shape[0], dtype=object)
            for k in range(cart.shape[0]):
                out[k] = Coordinates.from_cartesian(cart[k], weights=None if np.isnan(w[k]).all() else w[k])
            values[name] = out
        elif isinstance(kind, list) and kind[0] == "ndarray_list":
            values[name] = [arrays.pop(f"{name}/{i}") for i in range(int(kind[1]))]
    for name, a in arrays.items():
        if "/" in name:
            raise NotImplementedError(f"member '{name}/$ndarray' belongs to an encoding this reader does not know")
        values[name] = a
    return values
