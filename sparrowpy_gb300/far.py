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

The JSON object names them under "sparrowpy_gb300.encoding". Files with
other pyfar object members, such as the reference's own Coordinates
encoding, are refused with the member's name.
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


def read(filename):
    """Read a file written by write(), or a pyfar file holding only ndarray and builtin members."""
    values, arrays = {}, {}
    with zipfile.ZipFile(filename, "r") as z:
        for m in z.namelist():
            if m == _BUILTINS:
                values.update(json.loads(z.read(m).decode("utf-8")))
            elif m.endswith("/$ndarray"):
                arrays[m[:-len("/$ndarray")]] = _npy_load(z.read(m))
            else:
                raise NotImplementedError(f"member '{m}': only ndarray and builtin members can be read here")
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
