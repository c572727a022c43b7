"""Particles (SimpleParticles + ParticleRaster, tina/core/particle.py): shaded
spheres sharing the depth buffer with triangles, against the oracle -- particle
id, int32 depth and float depth bit-exact, RGB within 1e-4."""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina


def _pars(n, seed, rmin=0.02, rmax=0.15):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    rad = rng.uniform(rmin, rmax, n).astype(np.float32)
    col = rng.uniform(0.1, 1.0, (n, 3)).astype(np.float32)
    return pos, rad, col


def test_describe_particles():
    pars = tina.SimpleParticles(maxpars=100, radius=0.05)
    pos, rad, col = _pars(150, 0)
    pars.set_particles(pos)
    assert pars.get_npars() == 100 and float(pars.sizes[0]) == pytest.approx(0.05)
    scene = tina.Scene(32)
    scene.add_object(pars)
    sc, keep = scene.describe('cpu')
    from taichi_three_gb300 import _native as N
    assert sc.objects[0].mesh.kind == N.T3_MESH_PARTICLES and sc.objects[0].nfaces == 100


def _render_both(scene, oracle_mod):
    scene.render()
    torch.cuda.synchronize()
    o = oracle_mod.render(scene)
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
def test_particles_parity(cuda, oracle_mod, raster):
    pos, rad, col = _pars(400, 1)
    pars = tina.SimpleParticles()
    pars.set_particles(pos)
    pars.set_particle_radii(rad)
    pars.set_particle_colors(col)
    scene = tina.Scene(160, 120)
    scene.add_object(pars)  # default material: Diffuse(color=Input('color'))
    scene.engine.set_camera(tina.lookat(back=(0.5, 0.4, 3)), tina.perspective(60, 160 / 120))
    scene.raster_mode = raster
    fid = _render_both(scene, oracle_mod)
    assert len(np.unique(fid[fid >= 0])) > 100


@pytest.mark.gpu
@pytest.mark.parametrize('raster', ['direct', 'binned'])
def test_particles_with_triangles_and_pbr(cuda, oracle_mod, raster):
    arrays = tina.workloads.soup_arrays(3000, 4, median_sigma=0.08, log_sd=0.6)
    scene, _ = tina.workloads.soup_scene(ntri=3000, res=(128, 96), seed=4, nlights=3, arrays=arrays)
    pos, rad, col = _pars(200, 2, 0.03, 0.1)
    pars = tina.SimpleParticles()
    pars.set_particles(pos)
    pars.set_particle_radii(rad)
    pars.set_particle_colors(col)
    scene.add_object(pars, tina.PBR(basecolor='color', metallic=0.4, roughness=0.3))
    scene.raster_mode = raster
    fid = _render_both(scene, oracle_mod)
    assert (fid >= 3000).sum() > 300 and ((fid >= 0) & (fid < 3000)).sum() > 300


@pytest.mark.gpu
def test_particles_uncoloured_unclipped(cuda, oracle_mod):
    pos, rad, col = _pars(100, 3, 0.05, 0.2)
    pos[:, 2] *= 3.0  # some particles beyond the clip range
    pars = tina.SimpleParticles()
    pars.set_particles(pos)
    pars.set_particle_radii(rad)
    pars.set_particle_colors(col)
    for clipping in (True, False):
        scene = tina.Scene(96, clipping=clipping, coloring=False)
        scene.add_object(pars)
        scene.engine.set_camera(tina.lookat(back=(0, 0, 3)), tina.perspective(60, 1))
        _render_both(scene, oracle_mod)
