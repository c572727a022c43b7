"""MeshSmoothNormal (tina/mesh/norm.py:17-55): per-vertex normals of indexed
meshes.  The oracle's serial loop against a numpy restatement, the CUDA
sort-and-sum (t3_smooth_normals) against the oracle bit for bit, and renders
through the normals against the oracle."""
import os
import sys

import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden'))
import recipes  # noqa: E402


def _random_indexed(nverts, nfaces, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(nverts, 3)).astype(np.float32)
    f = rng.integers(0, nverts - 1, size=(nfaces, 3)).astype(np.int32)  # vertex nverts-1 unused
    f[::97, 1] = f[::97, 0]                                             # degenerate faces
    return v, f


def _numpy_smooth(v, f):
    """The reference loop in numpy float32 scalars (no fused operations)."""
    f32 = np.float32
    acc = np.zeros((len(v), 3), np.float32)

    def normalized(a):
        d = (a[0] * a[0] + a[1] * a[1]) + a[2] * a[2]
        inv = f32(1) / np.sqrt(f32(d))
        return np.array([inv * a[0], inv * a[1], inv * a[2]], np.float32)

    with np.errstate(all='ignore'):
        for i, j, k in f:
            a, b, c = v[i], v[j], v[k]
            e1, e2 = b - a, c - a
            cr = np.array([e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                           e1[0] * e2[1] - e1[1] * e2[0]], np.float32)
            n = normalized(cr)
            for x in (i, j, k):
                acc[x] = acc[x] + n
        return np.stack([normalized(a) for a in acc])


def _same(a, b):
    nan = np.isnan(a)
    return np.array_equal(nan, np.isnan(b)) and np.array_equal(a[~nan].view(np.uint32), b[~nan].view(np.uint32))


def test_oracle_matches_numpy_restatement(oracle_mod):
    v, f = _random_indexed(60, 150, 0)
    conn = tina.ConnectiveMesh()
    conn.set_vertices(v)
    conn.set_faces(f)
    m = N.t3_mesh()
    keep = []
    conn._t3_fill(m, 'cpu', keep)
    got = oracle_mod.smooth_normals(m, len(v))
    assert _same(got, _numpy_smooth(v, f))
    assert np.isnan(got[-1]).all()  # a vertex no face uses


def test_smooth_normal_wraps_indexed_meshes_only():
    with pytest.raises(NotImplementedError):
        tina.MeshSmoothNormal(tina.SimpleMesh())
    v, f = recipes._bumpy_sphere(1)
    model = tina.MeshSmoothNormal(tina.MeshModel(recipes._obj(v, f)))
    with pytest.raises(RuntimeError):
        model._t3_fill(N.t3_mesh(), 'cpu', [])  # no normals before pre_compute


@pytest.mark.gpu
def test_cuda_smooth_normals_bit_exact(cuda, oracle_mod):
    for nverts, nfaces, seed in ((50, 10, 1), (20_000, 150_000, 2), (3, 1, 3)):
        v, f = _random_indexed(nverts, nfaces, seed)
        conn = tina.ConnectiveMesh()
        conn.set_vertices(v)
        conn.set_faces(f)
        sm = tina.MeshSmoothNormal(conn)
        sm.update_normal()
        torch.cuda.synchronize()
        m = N.t3_mesh()
        keep = []
        host = tina.ConnectiveMesh()
        host.verts, host.faces, host.nfaces = torch.from_numpy(v), torch.from_numpy(f), len(f)
        host._t3_fill(m, 'cpu', keep)
        assert _same(sm.norm.cpu().numpy(), oracle_mod.smooth_normals(m, nverts)), (nverts, nfaces)


@pytest.mark.gpu
def test_smooth_render_parity_and_uncached_update(cuda, oracle_mod):
    v, f = recipes._bumpy_sphere(7, nlat=16, nlon=24)
    model = tina.MeshModel(recipes._obj(v, f))
    conn = tina.ConnectiveMesh()
    conn.set_vertices(v * np.float32(0.5))
    conn.set_faces(f)
    live = tina.MeshSmoothNormal(conn, cached=False)
    scene = tina.Scene(160, 120, smoothing=True)
    scene.add_object(tina.MeshSmoothNormal(model), tina.PBR(basecolor=[0.8, 0.6, 0.4], roughness=0.3))
    scene.add_object(tina.MeshTransform(live, tina.translate([0.7, 0.3, 0.5])), tina.Classic())
    scene.engine.set_camera(tina.lookat(back=(0.3, 0.2, 3)), tina.perspective(60, 160 / 120))
    for step in range(2):
        scene.render()
        torch.cuda.synchronize()
        o = oracle_mod.render(scene)
        assert np.array_equal(scene.face_id.cpu().numpy(), o['face_id'])
        assert np.array_equal(scene.engine.depth.cpu().numpy(), o['depth'])
        assert np.abs(scene.img.cpu().numpy() - o['rgb']).max() <= 1e-4
        assert (o['face_id'] >= len(f)).sum() > 200 and ((o['face_id'] >= 0) & (o['face_id'] < len(f))).sum() > 200
        # move the uncached mesh's vertices: its normals follow at the next render
        conn.set_vertices((v * np.float32(0.5)) * np.float32([1.0, 1.3, 0.8]))
