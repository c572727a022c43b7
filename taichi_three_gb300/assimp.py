"""Wavefront OBJ reading (tina/assimp/obj.py): readobj -> the dict MeshModel
takes ({'v', 'vt', 'vn', 'f'} numpy arrays, 'f' [n, 3, 3] 0-based v/vt/vn
indices per corner).

Behaviour kept from the reference so that face ids match: vertices, texture
and normal lines are read first, then faces; polygons are split into
triangles as (0,1,2),(2,3,0) for quads and a fan (0,n,n+1) beyond; a missing
index field is 0; empty arrays become one zero row; orient permutes and
negates axes (a leading '-' reverses each face's corner order); scale='auto'
centres and normalises.
"""
import io

import numpy as np


def _triangulate(faces, idx):
    if len(idx) == 3:
        faces.append(idx)
    elif len(idx) == 4:
        faces.append([idx[0], idx[1], idx[2]])
        faces.append([idx[2], idx[3], idx[0]])
    elif len(idx) > 4:
        for k in range(1, len(idx) - 1):
            faces.append([idx[0], idx[k], idx[k + 1]])
    else:
        raise ValueError(f'a face needs at least 3 corners, got {len(idx)}')


def _lines(path):
    if callable(getattr(path, 'readlines', None)):
        lines = path.readlines()
    elif isinstance(path, (bytes, bytearray)):
        lines = io.BytesIO(path).readlines()
    else:
        with open(path, 'rb') as f:
            lines = f.readlines()
    return [l if isinstance(l, bytes) else l.encode() for l in lines]


def readobj(path, orient='xyz', scale=None, simple=False, usemtl=True, quadok=False):
    """OBJ file (path, bytes or a file object) -> dict (tina/assimp/obj.py:17-94)."""
    lines = _lines(path)
    v, vt, vn, faces, mtls = [], [], [], [], []
    mtllib = None
    for line in lines:
        parts = line.strip().split(maxsplit=1)
        if len(parts) != 2:
            continue
        try:
            nums = [float(x) for x in parts[1].split()]
        except ValueError:
            continue
        {b'v': v, b'vt': vt, b'vn': vn}.get(parts[0], []).append(nums)
    for line in lines:
        parts = line.strip().split(maxsplit=1)
        if len(parts) != 2:
            continue
        kind, rest = parts[0], parts[1].split()
        if kind == b'mtllib':
            mtllib = rest[0]
        elif kind == b'usemtl':
            mtls.append([len(faces), rest[0]])
        elif kind == b'f':
            idx = [[int(x) - 1 if x else 0 for x in corner.split(b'/')] for corner in rest]
            if quadok:
                faces.append(idx)
            else:
                _triangulate(faces, idx)
    out = {
        'v': np.array(v, np.float32) if v else np.zeros((1, 3), np.float32),
        'vt': np.array(vt, np.float32) if vt else np.zeros((1, 2), np.float32),
        'vn': np.array(vn, np.float32) if vn else np.zeros((1, 3), np.float32),
        'f': np.array(faces, np.int32) if faces else np.zeros((1, 3, 3), np.int32),
    }
    if usemtl:
        out['usemtl'] = mtls
        out['mtllib'] = mtllib
    if orient is not None:
        objorient(out, orient)
    if scale is not None:
        if scale == 'auto':
            objautoscale(out)
        else:
            out['v'] *= scale
    if simple:
        return out['v'], out['f'][:, :, 0]
    return out


def objorient(obj, orient):
    """Axis permutation / negation, e.g. 'xZy' (tina/assimp/obj.py:187-205)."""
    flip = orient.startswith('-')
    if flip:
        orient = orient[1:]
    axes = ['xyz'.index(c.lower()) for c in orient]
    neg = [c.isupper() for c in orient]
    if axes != [0, 1, 2]:
        obj['v'][:, (0, 1, 2)] = obj['v'][:, tuple(axes)]
        obj['vn'][:, (0, 1, 2)] = obj['vn'][:, tuple(axes)]
    for i, n in enumerate(neg):
        if n:
            obj['v'][:, i] = -obj['v'][:, i]
            obj['vn'][:, i] = -obj['vn'][:, i]
    if flip:
        obj['f'] = np.ascontiguousarray(obj['f'][:, ::-1])


def objautoscale(obj):
    obj['v'] -= np.average(obj['v'], axis=0)
    obj['v'] /= np.max(np.abs(obj['v']))


def objverts(obj):
    return obj['v'][obj['f'][:, :, 0]]


def objnorms(obj):
    return obj['vn'][obj['f'][:, :, 2]]


def objcoors(obj):
    return obj['vt'][obj['f'][:, :, 1]]
