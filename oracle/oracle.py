"""Test infrastructure only: ctypes binding of oracle/_build/libtina_oracle.so.

`render(scene)` evaluates a taichi_three_gb300.Scene on the CPU with the
restatement in oracle/tina_oracle.cpp, from the same t3_scene descriptor the
CUDA library receives (its pointers placed on the host).
"""
import ctypes as C

import numpy as np

from . import build as _build

_lib = None


def load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = C.CDLL(path)
        f = lib.oracle_render_f32
        f.restype = C.c_int
        f.argtypes = [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 5
        f = lib.oracle_render_f64
        f.restype = C.c_int
        f.argtypes = [C.c_void_p, C.c_int, C.c_int] + [C.c_void_p] * 4
        lib.oracle_grid_normals.restype = C.c_int
        lib.oracle_grid_normals.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        lib.oracle_aces_f32.restype = C.c_int
        lib.oracle_aces_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        lib.oracle_max_threads.restype = C.c_int
        lib.oracle_smooth_normals.restype = C.c_int
        lib.oracle_smooth_normals.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
        lib.oracle_pixels_f64.restype = C.c_int
        lib.oracle_pixels_f64.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_uint32,
                                          C.c_int, C.c_void_p, C.c_void_p]
        lib.oracle_sample_ibl_f32.restype = C.c_int
        lib.oracle_sample_ibl_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                              C.c_void_p]
        lib.oracle_sample_leaf_f32.restype = C.c_int
        lib.oracle_sample_leaf_f32.argtypes = [C.c_int] + [C.c_void_p] * 5 + [C.c_int64, C.c_void_p,
                                                                             C.c_void_p]
        lib.oracle_mix_choice_f32.restype = C.c_int
        lib.oracle_mix_choice_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        lib.oracle_pixels_f32.restype = C.c_int
        lib.oracle_pixels_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int, C.c_void_p,
                                          C.c_void_p]
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def render_desc(sc, mode=0, nthreads=0, fp64=False, want_depth_f=True):
    """Renders a t3_scene descriptor (host pointers).  mode 0 = serial face order
    (the oracle), 1 = OpenMP packed-key minimum (the timed CPU baseline)."""
    lib = load()
    W, H = sc.frame.width, sc.frame.height
    out = {
        'rgb_pre': np.empty((W, H, 3), np.float32),
        'face_id': np.empty((W, H), np.int32),
        'depth': np.empty((W, H), np.int32),
    }
    if fp64:
        out['rgb'] = np.empty((W, H, 3), np.float64)
        rc = lib.oracle_render_f64(C.addressof(sc), mode, nthreads, _p(out['rgb']), _p(out['rgb_pre']),
                                   _p(out['face_id']), _p(out['depth']))
    else:
        out['rgb'] = np.empty((W, H, 3), np.float32)
        out['depth_f'] = np.empty((W, H), np.float32) if want_depth_f else None
        rc = lib.oracle_render_f32(C.addressof(sc), mode, nthreads, _p(out['rgb']), _p(out['rgb_pre']),
                                   _p(out['face_id']), _p(out['depth']), _p(out['depth_f']))
    if rc != 0:
        raise RuntimeError(f'oracle render failed ({rc})')
    return out


def render(scene, mode=0, nthreads=0, fp64=False, want_depth_f=True):
    """Renders a taichi_three_gb300.Scene with the oracle (runs the scene's mesh
    pre_compute on the host first, e.g. MeshGrid normals)."""
    for obj in scene.objects:
        pre_compute_host(obj)
    sc, keep = scene.describe('cpu')
    out = render_desc(sc, mode, nthreads, fp64, want_depth_f)
    del keep
    return out


def pixels_f64(scene, pixels, spp=0, seed=0, nthreads=0):
    """FP64 colours (pre, post tonemap) of the given pixel indices x*H + y, shaded
    over the FP32 raster's winners; spp > 0 overrides the IBL sample count and
    seed (the converged reference for error statements)."""
    lib = load()
    for obj in scene.objects:
        pre_compute_host(obj)
    sc, keep = scene.describe('cpu')
    px = np.ascontiguousarray(pixels, dtype=np.int64)
    pre = np.empty((len(px), 3), np.float64)
    post = np.empty((len(px), 3), np.float64)
    rc = lib.oracle_pixels_f64(C.addressof(sc), _p(px), len(px), int(spp), int(seed) & 0xFFFFFFFF,
                               int(nthreads), _p(pre), _p(post))
    if rc != 0:
        raise RuntimeError(f'oracle_pixels_f64 failed ({rc})')
    del keep
    return pre, post


def pixels_f32(scene, pixels, nthreads=0):
    """FP32 colours (after the tonemap when the scene has it) and winning face
    ids of the given pixel indices x*H + y, with the scene's own IBL sample
    stream: the oracle for sampled pixels of frames too large to shade whole."""
    lib = load()
    for obj in scene.objects:
        pre_compute_host(obj)
    sc, keep = scene.describe('cpu')
    px = np.ascontiguousarray(pixels, dtype=np.int64)
    rgb = np.empty((len(px), 3), np.float32)
    fid = np.empty(len(px), np.int32)
    rc = lib.oracle_pixels_f32(C.addressof(sc), _p(px), len(px), int(nthreads), _p(rgb), _p(fid))
    if rc != 0:
        raise RuntimeError(f'oracle_pixels_f32 failed ({rc})')
    del keep
    return rgb, fid


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def sample_ibl(material_desc, tables, idir, nrm):
    """material.sample_ibl(tab, idir, nrm) for n pairs (t3_material with constant
    parameters, t3_ibl_tables with host pointers) -> [n, 3]."""
    lib = load()
    idir, nrm = _f32(idir), _f32(nrm)
    out = np.empty((len(idir), 3), np.float32)
    rc = lib.oracle_sample_ibl_f32(C.addressof(material_desc), C.addressof(tables), _p(idir), _p(nrm),
                                   len(idir), _p(out))
    if rc != 0:
        raise RuntimeError(f'oracle_sample_ibl_f32 failed ({rc})')
    return out


def sample_leaf(op, param, f0, idir, nrm, xi):
    """One draw of a leaf sampler per row -> (direction [n, 3], weight [n, 3])."""
    lib = load()
    param, f0, idir, nrm, xi = _f32(param), _f32(f0), _f32(idir), _f32(nrm), _f32(xi)
    d = np.empty((len(idir), 3), np.float32)
    w = np.empty((len(idir), 3), np.float32)
    lib.oracle_sample_leaf_f32(int(op), _p(param), _p(f0), _p(idir), _p(nrm), _p(xi), len(idir), _p(d), _p(w))
    return d, w


def mix_choice(fac, xi):
    """MixMaterial.sample's branch choice -> (weight factor [n, 3], second child chosen [n])."""
    lib = load()
    fac, xi = _f32(fac), _f32(xi)
    w = np.empty((len(xi), 3), np.float32)
    pick = np.empty(len(xi), np.int32)
    lib.oracle_mix_choice_f32(_p(fac), _p(xi), len(xi), _p(w), _p(pick))
    return w, pick.astype(bool)


def grid_normals(pos):
    lib = load()
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    nrm = np.empty_like(pos)
    lib.oracle_grid_normals(_p(pos), _p(nrm), pos.shape[0], pos.shape[1])
    return nrm


def aces(x):
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty_like(x)
    lib.oracle_aces_f32(_p(x), _p(y), x.size)
    return y


def smooth_normals(mesh_desc, nverts):
    """MeshSmoothNormal's vertex normals of an indexed t3_mesh (host pointers)."""
    lib = load()
    out = np.empty((nverts, 3), np.float32)
    rc = lib.oracle_smooth_normals(C.addressof(mesh_desc), int(nverts), _p(out))
    if rc != 0:
        raise RuntimeError(f'oracle_smooth_normals failed ({rc})')
    return out


def pre_compute_host(obj):
    """The mesh's pre_compute on the CPU (MeshGrid normals, MeshSmoothNormal
    vertex normals) for meshes held in host memory; device meshes are left
    untouched."""
    node = obj
    while node is not None:
        if type(node).__name__ == 'MeshSmoothNormal' and not node.mesh.verts.is_cuda:
            import torch
            from taichi_three_gb300 import _native as N
            m = N.t3_mesh()
            keep = []
            node.mesh._t3_fill(m, 'cpu', keep)
            node.norm = torch.from_numpy(smooth_normals(m, int(node.mesh.verts.shape[0])))
        node = getattr(node, 'mesh', None)
    base = obj
    while hasattr(base, 'mesh') and not hasattr(base, 'res'):
        base = base.mesh
    if hasattr(base, 'auto_normals') and base.auto_normals and not base.pos.is_cuda:
        import torch
        base.nrm = torch.from_numpy(grid_normals(base.pos.numpy()))


def max_threads():
    return load().oracle_max_threads()
