"""t3_render_noalloc: one frame with no device allocation by the library.

Some callers cannot allocate device memory: a renderer running inside a host
application that owns the GPU's memory and only hands over its input and
output buffers (a plug-in or frame callback where cudaMalloc is forbidden or
could stall).  For them t3_render_noalloc renders a frame with its scratch in a
fixed array built into libtina3.so.  This test calls it through the C ABI on
two different scenes in a row and checks each frame against t3_render (the
entry point with a caller-allocated workspace): face id, depth and float depth
bit-exact, scene.img within the 1e-4 tolerance the parity tests use.  It lives
in its own file that pytest collects last, and passes alone or after the rest.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-4


def _scenes():
    verts, norms, attrs = tina.workloads.soup_arrays(5000, seed=21, median_sigma=0.05)
    a, _ = tina.workloads.soup_scene(ntri=5000, res=(320, 200), seed=21, nlights=5,
                                     arrays=(verts, norms, attrs))
    b, _ = tina.workloads.sphere_scene(256)
    b.lighting.add_light(pos=[1.0, 2.0, 2.5], color=[2.0, 1.5, 1.0])
    return [a, b]


def _outputs(W, H, dev):
    return {'rgb': torch.full((W, H, 3), -7.0, device=dev),
            'face_id': torch.full((W, H), -7, dtype=torch.int32, device=dev),
            'depth': torch.full((W, H), -7, dtype=torch.int32, device=dev),
            'depth_f': torch.full((W, H), -7.0, device=dev)}


def test_noalloc_render_matches_t3_render_on_two_calls(cuda):
    lib = N.load()
    dev = cuda
    scenes = _scenes()
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    outs_all = [_outputs(*s.res, dev) for s in scenes]
    descs = []
    for s in scenes:
        for obj in s.objects:
            obj.pre_compute()
        descs.append(s.describe(dev))
    # two no-alloc frames back to back (the second reuses the scratch the first left)
    for (sc, _keep), o in zip(descs, outs_all):
        outs = N.t3_outputs(o['rgb'].data_ptr(), o['face_id'].data_ptr(), o['depth'].data_ptr(),
                            o['depth_f'].data_ptr())
        rc = lib.t3_render_noalloc(C.byref(sc), status.data_ptr(), C.byref(outs), stream)
        assert rc == N.T3_OK
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    # the same frames through t3_render with its allocated workspace
    for s, o in zip(scenes, outs_all):
        s.render()
        torch.cuda.synchronize()
        assert np.array_equal(o['face_id'].cpu().numpy(), s.face_id.cpu().numpy())
        assert np.array_equal(o['depth'].cpu().numpy(), s.engine.depth.cpu().numpy())
        assert np.array_equal(o['depth_f'].cpu().numpy().view(np.uint32),
                              s.depth_f.cpu().numpy().view(np.uint32))
        err = np.abs(o['rgb'].cpu().numpy() - s.img.cpu().numpy()).max()
        assert err <= RGB_TOL, err
        assert (o['face_id'] >= 0).sum().item() > 1000


def _call_noalloc(lib, scene, dev, status):
    for obj in scene.objects:
        obj.pre_compute()
    sc, keep = scene.describe(dev)
    o = _outputs(*scene.res, dev)
    outs = N.t3_outputs(o['rgb'].data_ptr(), o['face_id'].data_ptr(), o['depth'].data_ptr(),
                        o['depth_f'].data_ptr())
    rc = lib.t3_render_noalloc(C.byref(sc), status.data_ptr(), C.byref(outs),
                               torch.cuda.current_stream().cuda_stream)
    assert rc == N.T3_OK
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in o.items()}


def _assert_same(got, scene):
    scene.render()
    torch.cuda.synchronize()
    assert np.array_equal(got['face_id'], scene.face_id.cpu().numpy())
    assert np.array_equal(got['depth'], scene.engine.depth.cpu().numpy())
    assert np.array_equal(got['depth_f'].view(np.uint32), scene.depth_f.cpu().numpy().view(np.uint32))
    ref = scene.img.cpu().numpy()
    ok = np.isfinite(ref)
    assert np.array_equal(np.isfinite(got['rgb']), ok)
    assert np.abs(got['rgb'][ok] - ref[ok]).max() <= RGB_TOL


def _mixed_scene():
    """Five objects sharing the scratch's large-face queue through per-object
    counters: a displaced MeshGrid, a ConnectiveMesh, a PBR soup with large
    faces, particles and a line soup."""
    scene = tina.Scene(256, 192, smoothing=True)
    grid = tina.MeshGrid((48, 40))
    x, y = grid.pos[..., 0], grid.pos[..., 1]
    grid.pos[..., 2] = 0.15 * torch.sin(6 * x) * torch.cos(5 * y)
    scene.add_object(grid, tina.PBR(metallic=0.3, roughness=0.4))
    sph = tina.PrimitiveMesh.sphere(lons=20, lats=10)
    v = sph.verts.cpu().numpy().reshape(-1, 3) * 0.5 + np.array([0.3, 0.2, 0.3], np.float32)
    conn = tina.ConnectiveMesh()
    conn.set_vertices(v)
    conn.set_vert_norms(sph.norms.cpu().numpy().reshape(-1, 3))
    conn.set_faces(np.arange(len(v)).reshape(-1, 3)[:, ::-1].copy())
    scene.add_object(conn, tina.Classic(color=[0.8, 0.5, 0.3]))
    verts, norms, attrs = tina.workloads.soup_arrays(400, seed=8, median_sigma=0.3)
    soup = tina.SimpleMesh()
    soup.set_face_verts(verts)
    soup.set_face_norms(norms)
    soup.set_face_attrs(attrs)
    scene.add_object(soup, tina.workloads.pbr_face_material())
    rng = np.random.default_rng(4)
    pars = tina.SimpleParticles()
    pars.set_particles(rng.uniform(-0.8, 0.8, (80, 3)).astype(np.float32))
    pars.set_particle_radii(rng.uniform(0.02, 0.06, 80).astype(np.float32))
    scene.add_object(pars, tina.Diffuse(color=0.7))
    lines = tina.SimpleMesh(npolygon=2)
    lines.set_face_verts(rng.uniform(-1, 1, (60, 2, 3)).astype(np.float32))
    scene.add_object(lines)
    scene.lighting.add_light(pos=[1.0, 2.0, 2.5], color=[2.0, 1.5, 1.0])
    scene.engine.set_camera(tina.lookat(back=(0.3, -1.2, 2.2)), tina.perspective(60, 256 / 192))
    return scene


def test_noalloc_multi_object_points_and_lines(cuda):
    """Grid and indexed vertex stages (which t3_render runs as a separate pass
    and the no-alloc frame folds into the raster), several objects, particles
    and lines: equal to t3_render on two calls in a row."""
    lib = N.load()
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    for _ in range(2):
        scene = _mixed_scene()
        got = _call_noalloc(lib, scene, cuda, status)
        assert int(status.item()) == 0
        ids = got['face_id']
        base = np.cumsum([0] + [scene.objects[o].raster.check_faces(o) for o in scene.objects])
        owners = np.searchsorted(base, ids[ids >= 0], side='right') - 1
        assert len(set(np.unique(owners).tolist())) >= 4  # the objects share the frame
        _assert_same(got, scene)


def test_noalloc_learned_ibl_frame(cuda):
    """The learned-IBL shading pass with no setup records (the no-alloc frame
    passes none): equal to t3_render's frame, which reads the raster's."""
    sky = tina.Skybox(tina.procedural_sky(32, seed=5))
    net = tina.IBLNet(seed=1)
    light = tina.SkyboxLighting(sky, mode='mlp', mlp=net)
    scene, _ = tina.workloads.soup_scene(ntri=3000, res=(160, 120), seed=4, nlights=0, ibl=True,
                                         lighting=light,
                                         arrays=tina.workloads.soup_arrays(3000, 4, median_sigma=0.05))
    lib = N.load()
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    got = _call_noalloc(lib, scene, cuda, status)
    assert int(status.item()) == 0
    assert (got['face_id'] >= 0).sum() > 2000
    _assert_same(got, scene)


def test_noalloc_large_face_queue_overflow(cuda):
    """More large faces (bbox above 4,096 px) than the built-in queue holds:
    the frame sets T3_STATUS_BIG_OVERFLOW and drops the excess, so every pixel
    keeps a face at least as deep as t3_render's winner (which sees them all)."""
    lib = N.load()
    n = int(N.T3_NOALLOC_MAX_BIG_FACES) + 4000
    W, H = 72, 60  # 4,320 px: every face below covers the frame
    z = np.linspace(0.2, 0.8, n, dtype=np.float64)
    tris = np.array([[(-40, -40), (200, -40), (-40, 200)]] * n, np.float64)
    from helpers import flat_scene
    scene, _ = flat_scene(tris, W=W, H=H, z=z[::-1].copy(), clipping=False)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    got = _call_noalloc(lib, scene, cuda, status)
    assert int(status.item()) & N.T3_STATUS_BIG_OVERFLOW
    assert (got['face_id'] >= 0).all()
    scene.render()
    torch.cuda.synchronize()
    ref = scene.engine.depth.cpu().numpy()
    assert (got['depth'] >= ref).all()
    assert (scene.face_id.cpu().numpy() == n - 1).all()  # the nearest face wins with every face seen


def test_noalloc_rejects_frames_beyond_its_scratch(cuda):
    lib = N.load()
    scene, _ = tina.workloads.sphere_scene(64)
    sc, keep = scene.describe(cuda)
    sc.frame.width, sc.frame.height = 2048, 2048  # 4 Mpx > T3_NOALLOC_MAX_PIXELS
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    img = torch.empty(4, device=cuda)
    outs = N.t3_outputs(img.data_ptr(), None, None, None)
    rc = lib.t3_render_noalloc(C.byref(sc), status.data_ptr(), C.byref(outs),
                               torch.cuda.current_stream().cuda_stream)
    assert rc == N.T3_ETOOBIG
