"""Animated grid captured as one CUDA graph (FrameGraph): every replayed frame
equals the same frame rendered eagerly, and the last frame matches the oracle
on the displaced positions."""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina

pytestmark = pytest.mark.gpu


def _grid_scene(raster='direct'):
    scene = tina.Scene(128, 96, smoothing=True, raster=raster)
    grid = tina.MeshGrid(64)
    scene.add_object(grid, tina.PBR(basecolor=(0.75, 0.62, 0.5), metallic=0.3, roughness=0.35))
    scene.lighting.clear_lights()
    scene.lighting.add_light(pos=[1.5, -1.0, 2.5], color=[3.0, 3.0, 3.0])
    scene.lighting.add_light(dir=[0.3, 0.5, 1.0], color=[0.8, 0.8, 0.8])
    scene.engine.set_camera(tina.lookat(back=(0.0, -1.6, 2.2)), tina.perspective(60, 128 / 96))
    return scene, grid


@pytest.mark.parametrize('raster', ['direct', 'binned'])
def test_frame_graph_equals_eager_frames(cuda, oracle_mod, raster):
    frames = 5
    scene, grid = _grid_scene(raster)
    eager = []
    for k in range(frames):
        grid.displace_wave(0.25 * k)
        scene.render()
        torch.cuda.synchronize()
        eager.append(scene.img.sum(dtype=torch.float64).item())
    last_eager = scene.img.cpu().numpy().copy()
    fg = tina.FrameGraph(scene, frames, update=lambda k: grid.displace_wave(0.25 * k)).capture()
    scene.img.zero_()
    fg.replay()
    torch.cuda.synchronize()
    assert fg.sums.cpu().numpy().tolist() == eager
    assert len(set(eager)) == frames  # the surface moves
    assert np.array_equal(scene.img.cpu().numpy(), last_eager)
    o = oracle_mod.render(scene)  # positions and normals of the last frame
    assert np.array_equal(scene.face_id.cpu().numpy(), o['face_id'])
    assert np.array_equal(scene.engine.depth.cpu().numpy(), o['depth'])
    assert np.abs(scene.img.cpu().numpy() - o['rgb']).max() <= 1e-4


def test_wave_grid_with_learned_ibl(cuda):
    sky = tina.Skybox(tina.procedural_sky(32, seed=1))
    net, _ = tina.train_for_skybox(sky, samples=1 << 15, spp=64, steps=50, batch=4096,
                                   irr_res=(32, 16), irr_spp=64)
    scene, grid = tina.workloads.wave_grid_scene(grid_res=96, res=(160, 90), skybox=sky, mlp=net)
    fg = tina.FrameGraph(scene, 4, update=lambda k: grid.displace_wave(0.5 * k)).capture()
    fg.replay()
    torch.cuda.synchronize()
    sums = fg.sums.cpu().numpy()
    assert np.isfinite(sums).all() and len(set(sums.tolist())) == 4
    assert scene.status() == 0
    assert (scene.face_id.cpu().numpy() >= 0).mean() > 0.2
