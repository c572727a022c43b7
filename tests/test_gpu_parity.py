"""GPU parity: the CUDA path through the C ABI against the oracle.

Bar (per the path's contract): triangle id, int32 depth and the float depth are
bit-exact with the serial FP32 restatement; shaded RGB (scene.img, after ACES)
agrees within 1e-4 max abs; every case also states its error against the FP64
oracle.
"""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from helpers import flat_scene, random_soup_scene

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-4  # max abs on scene.img


def gpu_render(scene):
    scene.render()
    torch.cuda.synchronize()
    return {
        'rgb': scene.img.cpu().numpy(),
        'face_id': scene.face_id.cpu().numpy(),
        'depth': scene.engine.depth.cpu().numpy(),
        'depth_f': scene.depth_f.cpu().numpy(),
    }


def assert_parity(g, o, rgb_tol=RGB_TOL, o64=None, hdr=False):
    """hdr: the image is not tonemapped (values unbounded), so the bound is
    relative: |gpu - oracle| <= rgb_tol * max(1, |oracle|)."""
    assert np.array_equal(g['face_id'], o['face_id']), \
        f"face id mismatch at {np.argwhere(g['face_id'] != o['face_id'])[:5].tolist()}"
    assert np.array_equal(g['depth'], o['depth'])
    assert np.array_equal(g['depth_f'].view(np.uint32), o['depth_f'].view(np.uint32))
    diff = np.abs(g['rgb'] - o['rgb'])
    if hdr:
        diff = diff / np.maximum(1.0, np.abs(o['rgb']))
    err = diff.max() if g['rgb'].size else 0.0
    assert err <= rgb_tol, f'rgb max {"rel" if hdr else "abs"} err {err}'
    if o64 is not None:
        same = g['face_id'] == o64['face_id']
        e64 = np.abs(g['rgb'][same] - o64['rgb'][same]).max() if same.any() else 0.0
        print(f'rgb err vs FP32 oracle {err:.3g}, vs FP64 oracle {e64:.3g} '
              f'({100 * (1 - same.mean()):.3f}% pixels differ in id)')
    return err


def test_sphere_512_lambert(cuda, oracle_mod):
    scene, mesh = tina.workloads.sphere_scene(512)
    g = gpu_render(scene)
    o = oracle_mod.render(scene)
    assert (o['face_id'] >= 0).sum() > 50000
    assert_parity(g, o, o64=oracle_mod.render(scene, fp64=True))


def test_sphere_default_lights_and_ambient(cuda, oracle_mod):
    scene = tina.Scene(256, smoothing=True)
    scene.add_object(tina.PrimitiveMesh.sphere(), tina.PBR(metallic=0.6, roughness=0.2))
    scene.engine.set_camera(tina.lookat(back=(0.5, 1.0, 3)), tina.perspective(45, 1))
    assert_parity(gpu_render(scene), oracle_mod.render(scene))


RASTERS = [dict(raster='direct'), dict(raster='binned', tile=8), dict(raster='binned', tile=16),
           dict(raster='binned', tile=32)]


@pytest.mark.parametrize('seed,material', [(1, 'pbr'), (2, 'classic'), (3, 'pbr'), (4, 'classic')])
@pytest.mark.parametrize('rast', RASTERS, ids=lambda r: '-'.join(map(str, r.values())))
def test_random_soups(cuda, oracle_mod, seed, material, rast):
    scene, _ = random_soup_scene(seed, ntri=3000, res=(160, 96), material=material, nlights=4,
                                 **rast)
    assert_parity(gpu_render(scene), oracle_mod.render(scene))


@pytest.mark.parametrize('rast', RASTERS[1:], ids=lambda r: 'tile%d' % r['tile'])
def test_binned_bins_overflow_then_grow(cuda, oracle_mod, rast):
    # 4-entry bins overflow; Scene.render sees the status bit and re-renders
    scene, _ = random_soup_scene(12, ntri=4000, res=(128, 96), bin_capacity=4, **rast)
    g = gpu_render(scene)
    assert scene.bin_capacity > 4
    assert_parity(g, oracle_mod.render(scene))
    assert not (scene.status() & tina._native.T3_STATUS_BIN_OVERFLOW)


@pytest.mark.parametrize('rast', RASTERS, ids=lambda r: '-'.join(map(str, r.values())))
def test_big_faces_and_multi_object_per_mode(cuda, oracle_mod, rast):
    scene, _ = flat_scene([[(-20, -20), (300, -20), (-20, 300)], [(5, 5), (200, 30), (40, 190)],
                           [(100, 100), (104, 101), (101, 106)]],
                          W=256, H=200, z=[0.6, 0.4, 0.3], clipping=False, **rast)
    assert_parity(gpu_render(scene), oracle_mod.render(scene))


@pytest.mark.parametrize('material', [
    lambda: tina.Lambert(), lambda: tina.Phong(shineness=12.5), lambda: tina.Phong(),
    lambda: tina.CookTorrance(roughness=0.3, fresnel=0.5), lambda: tina.Lamp(color=[0.3, 0.6, 0.9]),
    lambda: tina.Lambert() * [0.2, 0.4, 0.6] + tina.Emission() * 0.1,
    lambda: tina.MixMaterial(tina.Lambert(), tina.Phong(shineness=8), tina.Input('normal')),
    lambda: tina.PBR(basecolor=tina.Input('pos'), metallic=0.5, roughness=0.6),
])
def test_material_variants(cuda, oracle_mod, material):
    scene, _ = random_soup_scene(5, ntri=1500, res=(96, 96), nlights=2)
    obj = next(iter(scene.objects))
    scene.objects[obj].material = material()
    scene.lighting.set_ambient_light([0.05, 0.1, 0.02])
    scene.lighting.add_light(dir=[0.2, -1, 0.5], color=[0.5, 0.5, 0.5])
    assert_parity(gpu_render(scene), oracle_mod.render(scene))


@pytest.mark.parametrize('opts', [dict(tonemap=False), dict(culling=False), dict(clipping=False),
                                  dict(smoothing=False), dict(bgcolor=(0.1, 0.2, 0.3))])
def test_scene_options(cuda, oracle_mod, opts):
    scene, _ = random_soup_scene(6, ntri=2000, res=(128, 80), **opts)
    assert_parity(gpu_render(scene), oracle_mod.render(scene), hdr=not scene.tonemap)


def test_shared_edges_and_ties(cuda, oracle_mod):
    lower = [(0, 0), (8, 0), (0, 8)]
    upper = [(8, 0), (8, 8), (0, 8)]
    for tris in ([lower, upper], [upper, lower], [lower, lower, upper, upper]):
        scene, _ = flat_scene(tris)
        assert_parity(gpu_render(scene), oracle_mod.render(scene))


def test_empty_and_single_face_scenes(cuda, oracle_mod):
    scene, mesh = flat_scene([[(1, 1), (5, 1), (1, 5)]], W=13, H=7)
    assert_parity(gpu_render(scene), oracle_mod.render(scene))
    mesh.set_face_verts(np.zeros((0, 3, 3), np.float32))
    mesh.set_face_norms(np.zeros((0, 3, 3), np.float32))
    g = gpu_render(scene)
    assert (g['face_id'] == -1).all() and (g['depth'] == 2**30).all()


def test_large_faces_take_the_queue_path(cuda, oracle_mod):
    # screen-filling faces exceed the per-thread bbox threshold
    scene, _ = flat_scene([[(-20, -20), (300, -20), (-20, 300)], [(5, 5), (200, 30), (40, 190)]],
                          W=256, H=200, z=[0.6, 0.4], clipping=False)
    assert_parity(gpu_render(scene), oracle_mod.render(scene))


@pytest.mark.parametrize('rast', [RASTERS[0], RASTERS[2]], ids=['direct', 'binned16'])
def test_mesh_edits_and_multi_object(cuda, oracle_mod, rast):
    verts, norms, attrs = tina.workloads.soup_arrays(1200, 9, median_sigma=0.1)
    scene = tina.Scene(120, 90, smoothing=True, **rast)
    base = tina.SimpleMesh()
    base.set_face_verts(verts)
    base.set_face_norms(norms)
    base.set_face_attrs(attrs)
    t = tina.MeshTransform(base, tina.translate([0.3, -0.1, 0.2]) @ tina.scale([0.7, 1.1, 0.9]))
    scene.add_object(tina.MeshNoCulling(tina.MeshFlipNormal(tina.MeshFlipCulling(t))),
                     tina.workloads.pbr_face_material())
    other = tina.SimpleMesh()
    other.set_face_verts(verts[:500] * 0.8)
    other.set_face_norms(norms[:500])
    scene.add_object(tina.MeshFlatNormal(other), tina.Classic(color=[0.9, 0.3, 0.2]))
    scene.engine.set_camera(tina.lookat(back=(1, 1, 2.5)), tina.perspective(50, 120 / 90))
    g = gpu_render(scene)
    o = oracle_mod.render(scene)
    assert set(np.unique(o['face_id'] >= 2400)) == {False, True}
    assert_parity(g, o)


@pytest.mark.parametrize('res', [64, (80, 41), (33, 70)], ids=['square', 'wide', 'tall'])
def test_mesh_grid_with_device_normals(cuda, oracle_mod, res):
    """MeshGrid (square, and rectangular both ways) with its normals from
    pre_compute on the device."""
    grid = tina.MeshGrid(res)
    x, y = grid.pos[..., 0], grid.pos[..., 1]
    grid.pos[..., 2] = 0.1 * torch.sin(8 * x + 0.3) * torch.cos(8 * y + 0.39)
    scene = tina.Scene(200, 150, smoothing=True)
    scene.add_object(grid, tina.PBR(metallic=0.2, roughness=0.3))
    scene.engine.set_camera(tina.lookat(back=(0.4, -1.5, 2.0)), tina.perspective(60, 200 / 150))
    g = gpu_render(scene)  # computes normals on the device (MeshGrid.pre_compute)
    nrm_gpu = grid.nrm.cpu().numpy()
    nrm_cpu = oracle_mod.grid_normals(grid.pos.cpu().numpy())
    assert np.array_equal(nrm_gpu.view(np.uint32), nrm_cpu.view(np.uint32))
    o = oracle_mod.render(scene)  # the descriptor carries the device-computed normals
    assert_parity(g, o)
    assert (g['face_id'] >= 0).sum() > 5000
    assert g["face_id"].max() > 0.8 * grid.get_nfaces()  # the far cells are drawn too


def test_indexed_meshes(cuda, oracle_mod):
    sphere = tina.PrimitiveMesh.sphere(lons=24, lats=12)
    v = sphere.verts.cpu().numpy().reshape(-1, 3)
    n = sphere.norms.cpu().numpy().reshape(-1, 3)
    conn = tina.ConnectiveMesh()
    conn.set_vertices(v)
    conn.set_vert_norms(n)
    conn.set_faces(np.arange(len(v)).reshape(-1, 3)[:, ::-1].copy())
    model = tina.MeshModel({'v': v, 'vn': n, 'vt': np.zeros((1, 2)),
                            'f': np.stack([np.arange(len(v)).reshape(-1, 3),
                                           np.zeros((len(v) // 3, 3), int),
                                           np.arange(len(v)).reshape(-1, 3)], axis=2)})
    for mesh, opts in ((conn, dict(culling=False)), (model, {})):
        scene = tina.Scene(96, smoothing=True, **opts)
        scene.add_object(mesh, tina.Classic())
        scene.engine.set_camera(tina.lookat(), tina.perspective(60, 1))
        assert_parity(gpu_render(scene), oracle_mod.render(scene))


def _two_overlapping_soups(seed=11, res=(120, 90)):
    """Two PBR / Classic soups over the same region (each covers the other's
    pixels), the second with a MeshTransform, so the depth test across objects
    decides most covered pixels."""
    scene, a = random_soup_scene(seed, ntri=1500, res=res)
    v, n, at = tina.workloads.soup_arrays(1200, seed + 1, median_sigma=0.08, log_sd=0.6)
    b = tina.SimpleMesh()
    b.set_face_verts(v)
    b.set_face_norms(n)
    b.set_face_attrs(at)
    bt = tina.MeshTransform(b)
    bt.set_transform(tina.translate([0.05, -0.03, 0.1]))
    scene.add_object(bt, tina.workloads.classic_face_material())
    return scene, a, bt


def test_raster_protocol_two_objects(cuda, oracle_mod):
    """tina/scene/raster.py:177, :183-187 driven by hand: one depth clear, then
    set_object / render_occup / render_color per object.  The shared depth keys
    make the objects occlude each other: the frame's depth and ids equal
    Scene.render's and the oracle's bit for bit, the image within 1e-4."""
    scene, a, bt = _two_overlapping_soups()
    o = oracle_mod.render(scene)
    g = gpu_render(scene)
    nA = a.get_nfaces()
    both = (o['face_id'] >= 0)
    assert (o['face_id'] >= nA).sum() > 500 and (both & (o['face_id'] < nA)).sum() > 500
    eng = scene.engine
    W, H = scene.res
    img = torch.zeros((W, H, 3), device='cuda')
    eng.clear_depth()
    for k, (obj, info) in enumerate(scene.objects.items()):
        raster = tina.TriangleRaster(eng, smoothing=True)
        shader = tina.Shader(img, scene.lighting, info.material)
        raster.set_object(obj)
        raster.render_occup()
        occ = raster.occup.cpu().numpy()
        if k == 0:
            # the first object alone: its winners of an empty frame
            assert (occ >= 0).sum() > 0
        else:
            # the second object wins exactly the pixels the frame gives it
            assert np.array_equal(occ >= 0, o['face_id'] >= nA)
            assert np.array_equal(occ[occ >= 0] + nA, o['face_id'][occ >= 0])
        raster.render_color(shader)
    torch.cuda.synchronize()
    keys = eng.keys.cpu().numpy()
    ids = np.where(keys == -1, -1, keys & 0xFFFFFFFF).astype(np.int32)
    assert np.array_equal(ids, o['face_id'])
    assert np.array_equal(ids, g['face_id'])
    assert np.array_equal(eng.depth.cpu().numpy(), o['depth'])
    tina.ToneMapping(scene.res).apply(img)
    won = o['face_id'] >= 0
    assert np.abs(img.cpu().numpy()[won] - o['rgb'][won]).max() <= RGB_TOL
    assert np.abs(img.cpu().numpy()[won] - g['rgb'][won]).max() <= RGB_TOL


class _CallersRaster:
    """A rasteriser of the caller's own (add_object(raster=...)): it only
    forwards the three protocol methods to a TriangleRaster."""

    def __init__(self, engine, **options):
        self.inner = tina.TriangleRaster(engine, **options)

    def set_object(self, mesh):
        self.inner.set_object(mesh)

    def render_occup(self):
        self.inner.render_occup()

    def render_color(self, shader):
        self.inner.render_color(shader)


def test_scene_render_with_callers_raster(cuda, oracle_mod):
    """A raster passed to add_object makes Scene.render run the object loop of
    the protocol (clear, occup + color per object, background, tonemap); every
    output equals the oracle's at the GPU bar, particles included."""
    scene, a, bt = _two_overlapping_soups(seed=5)
    scene.objects[bt].raster = _CallersRaster(scene.engine, smoothing=True)
    rng = np.random.default_rng(3)
    pars = tina.SimpleParticles()
    pars.set_particles(rng.uniform(-0.8, 0.8, (60, 3)).astype(np.float32))
    pars.set_particle_radii(rng.uniform(0.02, 0.08, 60).astype(np.float32))
    scene.add_object(pars, tina.Diffuse(color=0.6))
    assert scene._foreign_rasters()
    o = oracle_mod.render(scene)
    g = gpu_render(scene)
    assert (o['face_id'] >= a.get_nfaces() + bt.get_nfaces()).sum() > 50  # particles win pixels
    assert_parity(g, o)


def test_tonemap_kernel(cuda, oracle_mod):
    x = torch.linspace(0, 20, 10001, device='cuda')
    y = x.clone()
    tina.ToneMapping(None).apply(y)
    ref = oracle_mod.aces(x.cpu().numpy())
    assert np.abs(y.cpu().numpy() - ref).max() < 1e-6


@pytest.mark.parametrize('rast', [RASTERS[0], RASTERS[2]], ids=['direct', 'binned16'])
def test_full_size_soup_1080p(cuda, oracle_mod, rast):
    """1,000,000-face PBR soup at 1920x1080 with 8 point lamps: bit-exact id and
    depth against the oracle (its OpenMP mode, which equals the serial one)."""
    scene, _ = tina.workloads.soup_scene(**rast)
    g = gpu_render(scene)
    o = oracle_mod.render(scene, mode=1)
    assert (o['face_id'] >= 0).mean() > 0.3
    assert_parity(g, o)
