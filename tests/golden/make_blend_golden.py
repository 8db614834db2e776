"""Meshes of the reference's .blend test files and the expected visibility of one of them.

The reference's tests/test_visibility.py:75-139 (test_vis_matrix_assembly,
skipped there without Blender) reads cube_simple.blend, cube.blend and
cube_blocked.blend through bpy and checks the patch-to-patch visibility of
each fine mesh against a known solution: every pair for cube_simple, the
pairs whose ray leaves patch i on its front side for cube, and the list A
of visible pairs written in the test file for cube_blocked.
tests/test_blender_import.py:9-16 checks the fine and rough meshes of
cube.blend.

This script reads the three files with the package's .blend reader
(sparrowpy_gb300.blend) and the list A from the test file as text, and
writes tests/golden/blend.npz: per file its vertices, faces (padded with
-1) and SHA-256, and A.

Usage:  python tests/golden/make_blend_golden.py [--ref /path/to/sparrowpy]
"""
import argparse
import ast
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from sparrowpy_gb300.blend import read_mesh  # noqa: E402

FILES = ("cube_simple", "cube", "cube_blocked")


def visible_pairs_of_test_file(path):
    """The literal list assigned to A in the reference's visibility test."""
    tree = ast.parse(open(path).read())
    for node in tree.body:
        if isinstance(node, ast.Assign) and any(getattr(t, "id", None) == "A" for t in node.targets):
            return np.array(ast.literal_eval(node.value), dtype=np.int32)
    raise ValueError(f"{path}: no list A")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref', default=os.environ.get('SPARROWPY_SRC'),
                    help='sparrowpy source tree (default: $SPARROWPY_SRC)')
    args = ap.parse_args()
    if not args.ref:
        ap.error('give --ref or set SPARROWPY_SRC')
    out = {}
    for name in FILES:
        path = os.path.join(args.ref, 'tests', 'test_data', name + '.blend')
        verts, faces = read_mesh(path)
        nv = max(len(f) for f in faces)
        conn = np.full((len(faces), nv), -1, dtype=np.int32)
        for i, f in enumerate(faces):
            conn[i, :len(f)] = f
        out[f'{name}_verts'] = verts
        out[f'{name}_faces'] = conn
        with open(path, 'rb') as fh:
            out[f'{name}_sha256'] = np.array(hashlib.sha256(fh.read()).hexdigest())
    out['cube_blocked_visible'] = visible_pairs_of_test_file(os.path.join(args.ref, 'tests', 'test_visibility.py'))
    np.savez_compressed(os.path.join(HERE, 'blend.npz'), **out)
    print({k: np.shape(v) for k, v in out.items()})


if __name__ == '__main__':
    main()
