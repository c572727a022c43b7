"""Raster edge cases: face id, int32 and float depth stay bit-exact with the
serial oracle where centres sit exactly on edges, edges are nearly parallel to
the pixel grid, faces are slivers, points or segments, corners lie ~10^4 px
off-screen or behind the camera.  These aim at what narrows the pixel tests
below the reference's bbox walk: the column-span walk (rows bounded per column
by the edge functions plus a margin) and the trimming of the walked range to
centres near the corners' [min, max].  Each scene runs through the direct and
binned rasters and the batched multi-view launch; faces whose pixels other
faces might win are also rendered one at a time."""
import os

import numpy as np
import pytest

import taichi_three_gb300 as tina

RASTERS = ['direct', 'binned']


def _ndc_scene(verts, res, **opts):
    """Faces given directly in NDC (identity camera), so viewport coordinates
    are chosen exactly."""
    scene = tina.Scene(res[0], res[1], **opts)
    mesh = tina.SimpleMesh()
    mesh.set_face_verts(np.asarray(verts, np.float32))
    scene.add_object(mesh)
    return scene


def _vp_to_ndc(px, py, res):
    return 2.0 * px / res[0] - 1.0, 2.0 * py / res[1] - 1.0


def centres_scene(**opts):
    """Right triangles whose edges run exactly through rows / columns of
    centres, and diagonals through centres (weights exactly 0 there)."""
    res = (96, 64)
    faces = []
    rng = np.random.default_rng(1)
    for _ in range(300):
        x0, y0 = rng.integers(0, 80) + 0.5, rng.integers(0, 50) + 0.5
        w, h = rng.integers(1, 12), rng.integers(1, 12)
        corners = [(x0, y0), (x0 + w, y0), (x0, y0 + h)] if rng.random() < 0.5 else \
                  [(x0, y0), (x0 + w, y0 + w), (x0, y0 + h)]
        z = rng.uniform(-0.9, 0.9)
        tri = [[*_vp_to_ndc(px, py, res), z] for px, py in corners]
        if rng.random() < 0.5:
            tri = tri[::-1]
        faces.append(tri)
    return _ndc_scene(faces, res, culling=False, **opts), 1000


def near_axis_scene(**opts):
    """Edges with slopes of 1e-7 .. 1e-2 against the pixel grid: their row
    bounds are ill-conditioned and must widen instead of cutting pixels."""
    res = (128, 96)
    rng = np.random.default_rng(2)
    faces = []
    for _ in range(400):
        x0, y0 = rng.uniform(4, 110), rng.uniform(4, 80)
        L = rng.uniform(2, 14)
        eps = 10.0 ** rng.uniform(-7, -2)
        if rng.random() < 0.5:
            corners = [(x0, y0), (x0 + eps, y0 + L), (x0 + L, y0 + rng.uniform(-L, L))]
        else:
            corners = [(x0, y0), (x0 + L, y0 + eps), (x0 + rng.uniform(-L, L), y0 + L)]
        z = rng.uniform(-0.9, 0.9, size=3)
        faces.append([[*_vp_to_ndc(px, py, res), zz] for (px, py), zz in zip(corners, z)])
    return _ndc_scene(faces, res, culling=False, **opts), 2000


def far_scene(**opts):
    """Slivers (two corners almost coincide), wedges with one corner ~10^4 px
    off-screen, a point face and a segment face."""
    rng = np.random.default_rng(3)
    faces = []
    for _ in range(200):
        a = rng.uniform(-1, 1, 2)
        b = a + rng.uniform(-0.3, 0.3, 2)
        c = b + rng.normal(0, 1e-5, 2)
        faces.append([[*a, 0.1], [*b, 0.2], [*c, 0.3]])
    for _ in range(100):
        a = rng.uniform(-0.9, 0.9, 2)
        b = a + rng.uniform(-0.1, 0.1, 2)
        c = rng.uniform(-150, 150, 2)
        faces.append([[*a, 0.0], [*b, 0.1], [*c, 0.5]])
    faces.append([[0.1, 0.1, 0.0], [0.1, 0.1, 0.0], [0.1, 0.1, 0.0]])
    faces.append([[-0.5, -0.5, 0.0], [0.0, 0.0, 0.0], [0.5, 0.5, 0.0]])
    return _ndc_scene(faces, (160, 120), culling=False, clipping=False, **opts), 500


def behind_scene(**opts):
    """Random faces around a perspective camera at z = 3, some with corners
    behind it (clip w of mixed sign)."""
    rng = np.random.default_rng(4)
    v = rng.uniform(-1.5, 1.5, size=(300, 3, 3)).astype(np.float32)
    v[:, :, 2] *= 2.5
    scene = tina.Scene(128, 96, culling=False, clipping=False, **opts)
    mesh = tina.SimpleMesh()
    mesh.set_face_verts(v)
    scene.add_object(mesh)
    scene.engine.set_camera(tina.lookat(back=(0, 0, 3)), tina.perspective(60, 128 / 96))
    return scene, 1000


SCENES = [centres_scene, near_axis_scene, far_scene, behind_scene]


def _compare(scene, oracle_mod):
    import torch
    torch.cuda.synchronize()
    o = oracle_mod.render(scene)
    fid = scene.face_id.cpu().numpy()
    assert np.array_equal(fid, o['face_id']), np.argwhere(fid != o['face_id'])[:5].tolist()
    assert np.array_equal(scene.engine.depth.cpu().numpy(), o['depth'])
    assert np.array_equal(scene.depth_f.cpu().numpy().view(np.uint32), o['depth_f'].view(np.uint32))
    return fid


def _check(scene, oracle_mod):
    scene.render()
    return _compare(scene, oracle_mod)


@pytest.mark.gpu
@pytest.mark.parametrize('raster', RASTERS)
@pytest.mark.parametrize('make', SCENES, ids=lambda f: f.__name__)
def test_edge_scene(cuda, oracle_mod, make, raster):
    scene, min_cover = make(raster=raster)
    fid = _check(scene, oracle_mod)
    assert (fid >= 0).sum() > min_cover


@pytest.mark.gpu
def test_edge_scenes_batched(cuda, oracle_mod):
    built = [make() for make in SCENES]
    b = tina.BatchRenderer([s for s, _ in built])
    b.render()
    assert b.status() == 0
    for scene, min_cover in built:
        assert (_compare(scene, oracle_mod) >= 0).sum() > min_cover


def _one_face_at_a_time(scene, mesh, faces, oracle_mod):
    """Renders each face alone (so no other face can win its pixels) and
    returns how many covered at least one pixel."""
    hits = 0
    for f in faces:
        mesh.set_face_verts(np.asarray(f, np.float32)[None])
        fid = _check(scene, oracle_mod)
        hits += bool((fid >= 0).any())
    return hits


@pytest.mark.gpu
@pytest.mark.parametrize('raster', RASTERS)
def test_wedges_with_a_far_corner_alone(cuda, oracle_mod, raster):
    # a short edge on screen and a corner 10^3..10^4 px away: the weights lose
    # about |p - c| |c - a| / |ab| * 2^-23 px to cancellation, so centres up to
    # ~1 px outside the corners' range can pass
    rng = np.random.default_rng(5)
    faces = []
    for _ in range(60):
        a = rng.uniform(-0.9, 0.9, 2)
        faces.append([[*a, 0.1], [*(a + rng.uniform(-0.1, 0.1, 2)), 0.2], [*rng.uniform(-150, 150, 2), 0.3]])
    scene = _ndc_scene(faces[:1], (160, 120), culling=False, clipping=False, raster=raster)
    assert _one_face_at_a_time(scene, list(scene.objects)[0], faces, oracle_mod) > 30


@pytest.mark.gpu
@pytest.mark.parametrize('raster', RASTERS)
def test_corners_behind_the_camera_alone(cuda, oracle_mod, raster):
    # clip w of mixed sign: the accepted region is not bounded by the corners'
    # viewport range, so such faces keep the reference's whole range
    scene, _ = behind_scene(raster=raster)
    mesh = list(scene.objects)[0]
    v = mesh.verts.cpu().numpy()
    behind = [f for f in v if (f[:, 2] > 3.0).any() and (f[:, 2] < 3.0).any()][:60]
    assert _one_face_at_a_time(scene, mesh, behind, oracle_mod) > 30


def _vp32(c, res):
    f32 = np.float32
    return f32(f32(f32(f32(c) * f32(0.5)) + f32(0.5)) * f32(res))


def _trimmed(lo, hi, T):
    """The setup's range of tested centres (t3_device.cuh tighten_to_centres),
    None where it keeps the reference's range."""
    f32 = np.float32
    mag = max(abs(lo), abs(hi))
    ext = f32(hi - lo)
    if not mag < 16777216:
        return None
    eps = f32(f32((2 + mag + ext) * f32(2.0 ** -16)) + f32(f32(T + 1) * f32(ext + 1) * f32(2.0 ** -18)))
    if not eps < 4:
        return None
    return int(np.ceil(f32(f32(lo - f32(0.5)) - eps))), int(np.floor(f32(f32(hi - f32(0.5)) + eps)))


def _column_rows(t, x, y0, y1):
    """Candidate rows [lo, hi] of column x (t3_raster.cuh column_consts and
    column_rows_c, as k_raster_direct runs them) in float32, with exact
    divisions where the kernel divides or takes reciprocals approximately (the
    margin's 2^-18 |B| term covers the difference)."""
    f32 = np.float32
    lo, hi = y0, y1
    S = f32(abs(t['bcnx']) + abs(t['bcny']) + abs(t['canx']) + abs(t['cany']))
    if not S < np.inf:
        return lo, hi
    bias = f32(0.5)
    px = f32(f32(x) + bias)
    ya, yb = f32(f32(y0) + bias), f32(f32(y1) + bias)
    dbx, dcx = abs(f32(px - t['bx'])), abs(f32(px - t['cx']))
    hb = max(abs(f32(ya - t['by'])), abs(f32(yb - t['by'])))
    hc = max(abs(f32(ya - t['cy'])), abs(f32(yb - t['cy'])))
    H = f32(hb + hc + abs(t['by']) + abs(t['cy']) + f32(2))
    N = f32(f32(f32(2) * f32(f32(dbx + dcx) + H)) * S + f32(4))
    A1 = f32(f32(f32(px - t['bx']) * t['bcny']) + f32(t['by'] * t['bcnx']))
    A2 = f32(f32(f32(px - t['cx']) * t['cany']) + f32(t['cy'] * t['canx']))
    A3 = f32(f32(f32(1) - A1) - A2)
    flo, fhi = f32(y0 - 1), f32(y1 + 1)
    for A, k in ((A1, f32(-t['bcnx'])), (A2, f32(-t['canx'])), (A3, f32(t['bcnx'] + t['canx']))):
        ak = abs(k)
        if not f32(ak * f32(1048576)) > S:
            continue
        B = f32(-A / k)
        m = f32(f32(f32(2.0 ** -18) * f32(f32(N / ak) + abs(B))) + f32(2.0 ** -20))
        if not (abs(B) < 1e30 and m < 1e30):
            continue
        if k > 0:
            lo = max(lo, int(np.ceil(min(max(f32(f32(B - m) - bias), flo), fhi))))
        else:
            hi = min(hi, int(np.floor(min(max(f32(f32(B + m) - bias), flo), fhi))))
    return lo, hi


def _adversarial_faces(rng, n, W, H):
    """Single faces in NDC (z 0.1 / 0.2 / 0.3): wedges with a far corner,
    slivers, long thin wedges, edges within 1e-8..1e-2 of the pixel axes,
    right triangles with edges through pixel centres, random faces."""
    for it in range(n):
        kind = it % 6
        a = rng.uniform(-0.9, 0.9, 2)
        if kind == 0:
            b, c = a + rng.uniform(-0.1, 0.1, 2), rng.uniform(-150, 150, 2)
        elif kind == 1:
            b = a + rng.uniform(-1, 1, 2)
            c = b + rng.normal(0, 10 ** rng.uniform(-7, -3), 2)
        elif kind == 2:
            b, c = a + rng.normal(0, 0.01, 2), a + rng.uniform(-8, 8, 2)
        elif kind == 3:
            L, e = rng.uniform(0.02, 0.2), 10 ** rng.uniform(-8, -2)
            if rng.random() < 0.5:
                b, c = a + [e, L], a + [L, rng.uniform(-L, L)]
            else:
                b, c = a + [L, e], a + [rng.uniform(-L, L), L]
        elif kind == 4:
            a = np.array([(rng.integers(0, W - 10) + 0.5) / W * 2 - 1, (rng.integers(0, H - 10) + 0.5) / H * 2 - 1])
            b, c = a + [rng.integers(1, 12) / W * 2, 0], a + [0, rng.integers(1, 12) / H * 2]
        else:
            b, c = rng.uniform(-1.2, 1.2, 2), rng.uniform(-1.2, 1.2, 2)
        yield np.array([[*a, 0.1], [*b, 0.2], [*c, 0.3]], np.float32)


# faces per seed; T3_SWEEP_FACES=20000 runs the large sweep
SWEEP_FACES = int(os.environ.get('T3_SWEEP_FACES', '600'))


@pytest.mark.parametrize('seed', [7, 8])
def test_narrowed_walks_hold_every_covered_centre(oracle_mod, seed):
    """The two bounds that narrow the pixel tests below the reference's bbox
    walk, restated in float32, against the oracle's coverage of single
    adversarial faces (identity camera, so every clip w is 1): the trimming of
    the walked range to centres near the corners' [min, max], and the
    column-span walk's candidate rows within that range."""
    f32 = np.float32
    W, H = 160, 120
    rng = np.random.default_rng(seed)
    scene = tina.Scene(W, H, culling=False, clipping=False)
    mesh = tina.SimpleMesh()
    mesh.set_face_verts(np.zeros((1, 3, 3), np.float32))
    scene.add_object(mesh)
    checked = 0
    for v in _adversarial_faces(rng, SWEEP_FACES, W, H):
        mesh.set_face_verts(v[None])
        pts = np.argwhere(oracle_mod.render(scene)['face_id'] == 0)
        if not len(pts):
            continue
        (ax, bx, cx), (ay, by, cy) = [_vp32(v[k, 0], W) for k in range(3)], [_vp32(v[k, 1], H) for k in range(3)]
        lx, hx, ly, hy = min(ax, bx, cx), max(ax, bx, cx), min(ay, by, cy), max(ay, by, cy)
        with np.errstate(all='ignore'):
            n = f32(f32(f32(bx - ax) * f32(cy - ay)) - f32(f32(by - ay) * f32(cx - ax)))
            t = dict(bx=bx, by=by, cx=cx, cy=cy, bcnx=f32(f32(bx - cx) / n), bcny=f32(f32(by - cy) / n),
                     canx=f32(f32(cx - ax) / n), cany=f32(f32(cy - ay) / n))
            S = f32(abs(t['bcnx']) + abs(t['bcny']) + abs(t['canx']) + abs(t['cany']))
            T = f32(f32(f32(hx - lx) + f32(hy - ly) + 4) * S)
            rng_x, rng_y = _trimmed(lx, hx, T), _trimmed(ly, hy, T)
            for axis, r in ((0, rng_x), (1, rng_y)):
                if r is not None:
                    assert pts[:, axis].min() >= r[0] and pts[:, axis].max() <= r[1], (axis, r, v.tolist())
            y0, y1 = max(int(np.floor(ly)), 0), min(int(np.ceil(hy)), H - 1)
            if rng_y is not None:
                y0, y1 = max(y0, rng_y[0]), min(y1, rng_y[1])
            for x in np.unique(pts[:, 0]):
                ys = pts[pts[:, 0] == x, 1]
                lo, hi = _column_rows(t, int(x), y0, y1)
                assert lo <= ys.min() and ys.max() <= hi, (int(x), lo, hi, ys.min(), ys.max(), v.tolist())
        checked += 1
    assert checked > SWEEP_FACES // 2


def test_edge_scenes_cover_on_the_oracle(oracle_mod):
    """The GPU cases' coverage floors hold on the oracle (no GPU needed)."""
    for make in SCENES:
        scene, min_cover = make()
        assert (oracle_mod.render(scene)['face_id'] >= 0).sum() > min_cover, make.__name__
