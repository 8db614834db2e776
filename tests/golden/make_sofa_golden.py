"""Arrays of the reference's SOFA test files, read with sparrowpy_gb300.sofa.

The reference's tests read three SOFA files (tests/test_data/ of sparrowpy):

* ITA_Dodecahedron.sofa, a FreeFieldDirectivityTF source directivity
  (tests/test_radiosity_sound_object.py:11-31, with the known answer
  get_directivity(...) = 0.0001908);
* ihta.E_sec_2.sofa and specular_gaussian5.sofa, GeneralTF directional
  scattering data of walls (tests/test_RadiosityDirectional.py).

The files cannot travel with the tests, so this script reads them with the
package's own HDF5 reader and stores what the tests use in
tests/golden/sofa.npz: the directivity's receiver positions and its data
for emitter 0 at the first four frequencies; the ihta file's frequencies,
positions and weights (its tests replace the data by ones); the specular
file whole; and, per file, its SHA-256 and the shape and sum of every
numeric variable, so that tests/test_sofa.py can check a re-read against
them when the reference tree is at hand.

Usage:  python tests/golden/make_sofa_golden.py [--ref /path/to/sparrowpy]
"""
import argparse
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from sparrowpy_gb300.sofa import read_sofa  # noqa: E402

FILES = ("ITA_Dodecahedron", "ihta.E_sec_2", "specular_gaussian5")


def digest(path):
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('SPARROWPY_SRC'),
                    help='sparrowpy source tree (default: $SPARROWPY_SRC)')
    args = ap.parse_args()
    if not args.ref:
        ap.error('give --ref or set SPARROWPY_SRC')
    data_dir = os.path.join(args.ref, 'tests', 'test_data')
    out = {}
    for name in FILES:
        path = os.path.join(data_dir, name + '.sofa')
        s = read_sofa(path)
        key = name.split('.')[0].lower()
        out[f'{key}_sha256'] = np.array(digest(path))
        stats = []
        for v in s.variables:
            a = getattr(s, v)
            if isinstance(a, np.ndarray) and a.dtype.kind in 'fiu':
                stats.append((v, list(a.shape), float(np.sum(a, dtype=np.float64))))
        out[f'{key}_stats'] = np.array(repr(stats))
        out[f'{key}_N'] = np.asarray(s.N)
        out[f'{key}_source_position'] = np.asarray(s.SourcePosition)
        out[f'{key}_source_type'] = np.array(s.SourcePosition_Type)
        out[f'{key}_receiver_position'] = np.asarray(s.ReceiverPosition)
        out[f'{key}_receiver_type'] = np.array(s.ReceiverPosition_Type)
        out[f'{key}_data_shape'] = np.array(np.shape(s.Data_Real))
        if hasattr(s, 'SourceWeights'):
            out[f'{key}_source_weights'] = np.asarray(s.SourceWeights)
            out[f'{key}_receiver_weights'] = np.asarray(s.ReceiverWeights)
    d = read_sofa(os.path.join(data_dir, 'ITA_Dodecahedron.sofa'))
    out['ita_dodecahedron_data0'] = (np.asarray(d.Data_Real)[0] + 1j * np.asarray(d.Data_Imag)[0])[:, :4]
    g = read_sofa(os.path.join(data_dir, 'specular_gaussian5.sofa'))
    out['specular_gaussian5_data'] = np.asarray(g.Data_Real) + 1j * np.asarray(g.Data_Imag)
    np.savez_compressed(os.path.join(HERE, 'sofa.npz'), **out)
    print({k: np.shape(v) for k, v in out.items()})


if __name__ == '__main__':
    main()
