"""Wavefront OBJ reading (tina/assimp/obj.py): readobj -> the dict MeshModel
takes ({'v', 'vt', 'vn', 'f'} numpy arrays, 'f' [n, 3, 3] 0-based v/vt/vn
indices per corner).

Behaviour kept from the reference so that face ids match: faces in file
order, polygons split into triangles as (0,1,2),(2,3,0) for quads and the fan
(0,k,k+1) otherwise; attribute rows whose fields are not all numbers are
skipped; a missing index field is 0; empty arrays become one zero row; orient
permutes and negates axes (a leading '-' reverses each face's corner order);
scale='auto' centres and normalises.
"""
import io

import numpy as np


def _split_polygon(corners):
    """The triangles of one face in the reference's order (face ids follow
    it): a quad as (0, 1, 2), (2, 3, 0), any other polygon as the fan
    (0, k, k + 1)."""
    n = len(corners)
    if n < 3:
        raise ValueError(f'a face needs at least 3 corners, got {n}')
    if n == 4:
        return [[corners[0], corners[1], corners[2]], [corners[2], corners[3], corners[0]]]
    return [[corners[0], corners[k], corners[k + 1]] for k in range(1, n - 1)]


def _lines(path):
    if callable(getattr(path, 'readlines', None)):
        lines = path.readlines()
    elif isinstance(path, (bytes, bytearray)):
        lines = io.BytesIO(path).readlines()
    else:
        with open(path, 'rb') as f:
            lines = f.readlines()
    return [l if isinstance(l, bytes) else l.encode() for l in lines]


def _floats(words):
    try:
        return [float(w) for w in words]
    except ValueError:
        return None


def readobj(path, orient='xyz', scale=None, simple=False, usemtl=True, quadok=False):
    """OBJ file (path, bytes or a file object) -> dict (tina/assimp/obj.py:17-94).

    One pass over the lines: `v` / `vt` / `vn` rows whose fields all parse as
    numbers, `f` corners as 0-based v/vt/vn triples (a missing field is 0),
    `usemtl` as [first face, name], the last `mtllib`; lines of one word are
    skipped."""
    attrs = {b'v': [], b'vt': [], b'vn': []}
    faces, mtls, mtllib = [], [], None
    for line in _lines(path):
        words = line.split()
        if len(words) < 2:
            continue
        kind, rest = words[0], words[1:]
        if kind in attrs:
            nums = _floats(rest)
            if nums is not None:
                attrs[kind].append(nums)
        elif kind == b'f':
            corners = [[int(x) - 1 if x else 0 for x in w.split(b'/')] for w in rest]
            faces.extend([corners] if quadok else _split_polygon(corners))
        elif kind == b'usemtl':
            mtls.append([len(faces), rest[0]])
        elif kind == b'mtllib':
            mtllib = rest[0]

    def table(rows, width, dtype):
        return np.array(rows, dtype) if rows else np.zeros((1, width), dtype)

    out = {'v': table(attrs[b'v'], 3, np.float32), 'vt': table(attrs[b'vt'], 2, np.float32),
           'vn': table(attrs[b'vn'], 3, np.float32),
           'f': np.array(faces, np.int32) if faces else np.zeros((1, 3, 3), np.int32)}
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
    """Reorients positions and normals in place, e.g. 'xZy': output axis i
    takes input axis orient[i], negated where the letter is upper case; a
    leading '-' also reverses every face's corner order
    (tina/assimp/obj.py:187-205)."""
    reverse = orient.startswith('-')
    spec = orient[1:] if reverse else orient
    src = ['xyz'.index(c.lower()) for c in spec]
    sign = np.array([-1.0 if c.isupper() else 1.0 for c in spec], np.float32)  # exact in float32
    for key in ('v', 'vn'):
        obj[key][:] = obj[key][:, src] * sign
    if reverse:
        obj['f'] = np.ascontiguousarray(obj['f'][:, ::-1])


def objautoscale(obj):
    """Centres the positions on their mean and scales the largest coordinate
    magnitude to 1."""
    v = obj['v']
    v -= v.mean(axis=0)
    v /= np.abs(v).max()


def objverts(obj):
    return obj['v'][obj['f'][:, :, 0]]


def objnorms(obj):
    return obj['vn'][obj['f'][:, :, 2]]


def objcoors(obj):
    return obj['vt'][obj['f'][:, :, 1]]
