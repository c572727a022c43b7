"""Wireframes (WireframeRaster, tina/core/wireframe.py; MeshToWire,
tina/mesh/wire.py; SimpleMesh(npolygon=2)): one-pixel DDA lines in the shared
depth buffer, against the oracle -- line id, int32 depth and float depth
bit-exact, RGB within 1e-4 (line pixels carry the raster's line colour)."""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N


def _lines(n, seed, spread=1.2, zscale=0.5):
    rng = np.random.default_rng(seed)
    ends = rng.uniform(-spread, spread, (n, 2, 3)).astype(np.float32)
    ends[:, :, 2] *= zscale
    return ends


def test_describe_wires():
    verts, _, _ = tina.workloads.soup_arrays(50, 0)
    mesh = tina.SimpleMesh()
    mesh.set_face_verts(verts)
    wire = tina.MeshToWire(mesh)
    assert wire.get_npolygon() == 2 and wire.get_nfaces() == 150
    lines = tina.SimpleMesh(npolygon=2)
    lines.set_face_verts(_lines(20, 1))
    assert lines.get_npolygon() == 2 and lines.get_nfaces() == 20
    with pytest.raises(ValueError):
        lines.set_face_verts(np.zeros((3, 3, 3), np.float32))
    scene = tina.Scene(32, linecolor=(0.1, 0.2, 0.3), clipping=True)
    scene.add_object(mesh)
    scene.add_object(wire)
    scene.add_object(tina.MeshTransform(lines, tina.translate([0, 0, 0.1])))
    assert isinstance(scene.objects[wire].raster, tina.WireframeRaster)
    assert isinstance(scene.objects[mesh].raster, tina.TriangleRaster)
    sc, keep = scene.describe('cpu')
    assert sc.frame.flags & N.T3_WIRE_CLIPPING
    assert [round(c, 6) for c in sc.frame.linecolor] == [0.1, 0.2, 0.3]
    assert sc.objects[1].mesh.flags & N.T3_MESH_WIREFRAME and sc.objects[1].nfaces == 150
    assert sc.objects[2].mesh.kind == N.T3_MESH_LINES and sc.objects[2].nfaces == 20
    assert sc.objects[2].mesh.flags == N.T3_MESH_TRANSFORM
    assert (sc.objects[1].face_base, sc.objects[2].face_base) == (50, 200)
    # an edge order flip around the wireframe is not a wireframe of the flipped mesh
    with pytest.raises(NotImplementedError):
        tina.MeshNoCulling(tina.MeshToWire(mesh))._t3_fill(N.t3_mesh(), 'cpu', [])



def test_describe_quad_grid_wires():
    # MeshGrid(as_quad=True) (grid.py:23-44): one quad per cell, four lines each under MeshToWire
    quads = tina.MeshGrid(5, as_quad=True)
    assert quads.get_npolygon() == 4 and quads.get_nfaces() == 16
    assert tina.MeshGrid(5).get_nfaces() == 32
    wire = tina.MeshToWire(tina.MeshTransform(quads, tina.translate([0, 0, 0.2])))
    assert wire.get_npolygon() == 2 and wire.get_nfaces() == 64
    scene = tina.Scene(32)
    scene.add_object(wire)
    sc, _ = scene.describe('cpu')
    m = sc.objects[0].mesh
    assert m.kind == N.T3_MESH_GRID and sc.objects[0].nfaces == 64 and m.nfaces == 16
    assert m.flags == N.T3_MESH_QUADS | N.T3_MESH_TRANSFORM | N.T3_MESH_WIREFRAME

def test_default_wire_options():
    scene = tina.Scene(16)
    lines = tina.SimpleMesh(npolygon=2)
    lines.set_face_verts(_lines(4, 2))
    scene.add_object(lines)
    sc, _ = scene.describe('cpu')
    assert not (sc.frame.flags & N.T3_WIRE_CLIPPING)          # WireframeRaster(clipping=False)
    assert sc.frame.flags & N.T3_CLIPPING                      # TriangleRaster(clipping=True)
    assert np.allclose(list(sc.frame.linecolor), [0.9, 0.6, 0.0])


def _render_both(scene, oracle_mod, mode=0):
    scene.render()
    torch.cuda.synchronize()
    o = oracle_mod.render(scene, mode=mode)
    fid = scene.face_id.cpu().numpy()
    assert np.array_equal(fid, o['face_id'])
    assert np.array_equal(scene.engine.depth.cpu().numpy(), o['depth'])
    assert np.array_equal(scene.depth_f.cpu().numpy().view(np.uint32), o['depth_f'].view(np.uint32))
    g = scene.img.cpu().numpy()
    ok = np.isfinite(o['rgb'])
    assert np.array_equal(np.isfinite(g), ok)
    assert np.abs(g[ok] - o['rgb'][ok]).max() <= 1e-4
    return fid


@pytest.mark.gpu
@pytest.mark.parametrize('raster', ['direct', 'binned'])
def test_wireframe_over_soup(cuda, oracle_mod, raster):
    arrays = tina.workloads.soup_arrays(4000, 5, median_sigma=0.06, log_sd=0.6)
    scene, mesh = tina.workloads.soup_scene(ntri=4000, res=(200, 150), seed=5, nlights=2, arrays=arrays)
    wire = tina.MeshToWire(mesh)
    scene.add_object(wire)
    scene.raster_mode = raster
    fid = _render_both(scene, oracle_mod)
    assert (fid >= 4000).sum() > 2000 and ((fid >= 0) & (fid < 4000)).sum() > 2000


@pytest.mark.gpu
def test_lines_clipping_and_far_endpoints(cuda, oracle_mod):
    ends = _lines(600, 6, spread=3.0, zscale=1.5)
    ends[:20, 1] = ends[:20, 0]                         # zero-length lines
    ends[20:40, 1] = ends[20:40, 0] + 1e-3              # under a pixel: one step with 0/0 weights
    ends[40:60, :, 0] *= 40.0                           # far outside the frame on both sides
    lines = tina.SimpleMesh(npolygon=2)
    lines.set_face_verts(ends)
    for clipping in (False, True):
        scene = tina.Scene(180, 130, clipping=clipping, linecolor=(0.3, 1.0, 0.2), bgcolor=0.1)
        scene.add_object(lines)
        scene.engine.set_camera(tina.lookat(back=(0.2, 0.1, 3)), tina.perspective(60, 180 / 130))
        fid = _render_both(scene, oracle_mod)
        assert (fid >= 0).sum() > 3000


@pytest.mark.gpu
@pytest.mark.parametrize('raster', ['direct', 'binned'])
def test_wire_of_edited_and_indexed_meshes(cuda, oracle_mod, raster):
    # MeshToWire over MeshNoCulling (doubled faces, odd copies reversed), over
    # an indexed mesh, over a grid, and a transform outside a line soup
    verts, _, _ = tina.workloads.soup_arrays(300, 7, median_sigma=0.1)
    soup = tina.SimpleMesh()
    soup.set_face_verts(verts)
    sphere = tina.PrimitiveMesh.sphere(lons=16, lats=10)
    v = sphere.verts.cpu().numpy().reshape(-1, 3)
    uniq, inv = np.unique(v.round(6), axis=0, return_inverse=True)
    conn = tina.ConnectiveMesh()
    conn.set_vertices(uniq.astype(np.float32))
    conn.set_faces(inv.reshape(-1, 3).astype(np.int32))
    grid = tina.MeshGrid(12)
    lines = tina.SimpleMesh(npolygon=2)
    lines.set_face_verts(_lines(50, 8))
    scene = tina.Scene(160, 120, smoothing=False)
    scene.add_object(tina.MeshToWire(tina.MeshNoCulling(soup)))
    scene.add_object(tina.MeshToWire(tina.MeshTransform(conn, tina.scale([0.5, 0.5, 0.5]))))
    scene.add_object(tina.MeshToWire(tina.MeshTransform(grid, tina.translate([0, 0, 0.3]))))
    scene.add_object(tina.MeshTransform(lines, tina.translate([0.1, 0.0, 0.2])))
    scene.add_object(tina.MeshToWire(lines))
    scene.add_object(grid)
    scene.engine.set_camera(tina.lookat(back=(0.3, 0.4, 2.6)), tina.perspective(60, 160 / 120))
    scene.raster_mode = raster
    fid = _render_both(scene, oracle_mod)
    sc, _ = scene.describe()
    bases = [sc.objects[o].face_base for o in range(sc.nobjects)] + [2 ** 31]
    for o in range(sc.nobjects):
        assert ((fid >= bases[o]) & (fid < bases[o + 1])).sum() > 20, o


@pytest.mark.gpu
@pytest.mark.parametrize('raster', ['direct', 'binned'])
def test_wires_under_ibl(cuda, oracle_mod, raster):
    # lines under the skybox lighting keep their colour; the sky fills the rest
    scene, mesh = tina.workloads.ibl_soup_scene(ntri=500, res=(96, 72), seed=9, env_res=32, spp=8,
                                                arrays=tina.workloads.soup_arrays(500, 9, median_sigma=0.1))
    scene.add_object(tina.MeshToWire(mesh))
    scene.raster_mode = raster
    _render_both(scene, oracle_mod, mode=1)


@pytest.mark.gpu
def test_wires_large_property(cuda, oracle_mod):
    # 300k lines at 1920x1080 against the OpenMP oracle: depth and ids bit-exact
    ends = _lines(300_000, 10, spread=1.5)
    lines = tina.SimpleMesh(npolygon=2)
    lines.set_face_verts(ends)
    scene = tina.Scene(1920, 1080)
    scene.add_object(lines)
    scene.engine.set_camera(tina.lookat(back=(0, 0, 3)), tina.perspective(60, 1920 / 1080))
    scene.render()
    torch.cuda.synchronize()
    o = oracle_mod.render(scene, mode=1, want_depth_f=False)
    assert np.array_equal(scene.face_id.cpu().numpy(), o['face_id'])
    assert np.array_equal(scene.engine.depth.cpu().numpy(), o['depth'])


@pytest.mark.gpu
def test_wires_and_particles_batched(cuda, oracle_mod):
    # one batched launch over a soup with its wireframe, a line soup and a
    # particle scene: each view against the oracle at the parity bar
    arrays = tina.workloads.soup_arrays(2000, 12, median_sigma=0.08, log_sd=0.6)
    soup, mesh = tina.workloads.soup_scene(ntri=2000, res=(128, 96), seed=12, nlights=2, arrays=arrays)
    soup.add_object(tina.MeshToWire(mesh))
    lines = tina.SimpleMesh(npolygon=2)
    lines.set_face_verts(_lines(400, 13))
    wires = tina.Scene(96, 80, linecolor=(0.2, 0.9, 0.4))
    wires.add_object(lines)
    wires.engine.set_camera(tina.lookat(back=(0.2, 0.1, 3)), tina.perspective(60, 96 / 80))
    rng = np.random.default_rng(14)
    pars = tina.SimpleParticles()
    pars.set_particles(rng.uniform(-1, 1, (300, 3)).astype(np.float32))
    pars.set_particle_radii(rng.uniform(0.03, 0.12, 300).astype(np.float32))
    pars.set_particle_colors(rng.uniform(0.2, 1, (300, 3)).astype(np.float32))
    balls = tina.Scene(100, 90)
    balls.add_object(pars)
    balls.engine.set_camera(tina.lookat(back=(0.3, 0.2, 3)), tina.perspective(60, 100 / 90))
    views = [soup, wires, balls]
    b = tina.BatchRenderer(views)
    b.render()
    assert b.status() == 0
    for scene in views:
        torch.cuda.synchronize()
        o = oracle_mod.render(scene)
        fid = scene.face_id.cpu().numpy()
        assert np.array_equal(fid, o['face_id'])
        assert np.array_equal(scene.engine.depth.cpu().numpy(), o['depth'])
        assert np.array_equal(scene.depth_f.cpu().numpy().view(np.uint32), o['depth_f'].view(np.uint32))
        assert np.abs(scene.img.cpu().numpy() - o['rgb']).max() <= 1e-4
        assert (fid >= 0).sum() > 1000
    fid = soup.face_id.cpu().numpy()
    assert (fid >= 2000).sum() > 500 and ((fid >= 0) & (fid < 2000)).sum() > 500


@pytest.mark.gpu
@pytest.mark.parametrize('raster', ['direct', 'binned'])
def test_quad_grid_wires(cuda, oracle_mod, raster):
    grid = tina.MeshGrid(12, as_quad=True)
    p = grid.pos.cpu().numpy()
    p[..., 2] = 0.2 * np.sin(3 * p[..., 0] + 0.3) * np.cos(2 * p[..., 1])
    grid.pos.copy_(torch.from_numpy(p).to(grid.pos.device))
    surface = tina.MeshGrid(16)
    scene = tina.Scene(150, 110, smoothing=True)
    scene.add_object(tina.MeshToWire(tina.MeshTransform(grid, tina.translate([0.1, 0.0, 0.15]))))
    scene.add_object(surface, tina.Classic())
    scene.engine.set_camera(tina.lookat(back=(0.3, -1.1, 2.3)), tina.perspective(60, 150 / 110))
    scene.raster_mode = raster
    fid = _render_both(scene, oracle_mod)
    nlines = 11 * 11 * 4
    wires = fid[(fid >= 0) & (fid < nlines)]
    assert len(wires) > 1000 and set((wires % 4).tolist()) == {0, 1, 2, 3}
    # a quad is not a face of the triangle raster
    bad = tina.Scene(32)
    bad.add_object(tina.MeshGrid(4, as_quad=True))
    with pytest.raises(RuntimeError):
        bad.render()
