"""SkyboxLighting's prefiltered lookup on the GPU (mode 'prefiltered', the
reference's default SkyboxLighting, tina/core/lighting.py:5-21): the tables
are baked on the device (t3_ibl_bake), then every frame reads them per
pixel.  Bar: face id / depth bit-exact, scene.img within 1e-4 of the oracle
given the same tables (the oracle's lookup is pinned to the reference's own
sample_ibl by tests/test_ibl_golden.py); a white furnace returns the sky
exactly through every table; Phong is refused as the reference refuses it.
"""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from helpers import random_soup_scene

pytestmark = pytest.mark.gpu


def _render(scene):
    scene.render()
    torch.cuda.synchronize()
    return {'rgb': scene.img.cpu().numpy(), 'face_id': scene.face_id.cpu().numpy(),
            'depth': scene.engine.depth.cpu().numpy()}


def test_white_furnace_through_the_tables(cuda):
    sky = tina.PlainSkybox((1.0, 1.0, 1.0))
    light = tina.SkyboxLighting(sky, precision=4)
    scene = tina.Scene(96, ibl=True, tonemap=False, lighting=light)
    scene.add_object(tina.PrimitiveMesh.sphere(), tina.Diffuse(color=1.0))
    g = _render(scene)
    tabs = light.ibltab
    for m in tabs.spec[1:] + [tabs.diffuse]:
        # every average of a constant sky is the sky (up to the bilerp weights' rounding)
        assert (m - 1.0).abs().max().item() < 2e-6
    covered = g['face_id'] >= 0
    assert covered.sum() > 1000 and (~covered).sum() > 1000
    assert np.abs(g['rgb'] - 1.0).max() < 4e-6


@pytest.mark.parametrize('material', ['pbr', 'mix'])
@pytest.mark.parametrize('raster', ['direct', 'binned'])
def test_prefiltered_frame_matches_oracle(cuda, oracle_mod, material, raster):
    sky = tina.Skybox(tina.procedural_sky(48, seed=2))
    light = tina.SkyboxLighting(sky, precision=8, seed=3)
    scene, mesh = random_soup_scene(4, ntri=1500, res=(128, 96), material='pbr', nlights=0, ibl=True,
                                    lighting=light, raster=raster)
    if material == 'mix':
        obj = next(iter(scene.objects))
        scene.objects[obj].material = tina.MixMaterial(
            tina.Lambert() * tina.FaceAttr(0, 3), tina.CookTorrance(roughness=tina.FaceAttr(3), fresnel=0.4),
            tina.Input('normal')) + tina.Emission() * 0.05
    g = _render(scene)
    o = oracle_mod.render(scene)
    assert np.array_equal(g['face_id'], o['face_id'])
    assert np.array_equal(g['depth'], o['depth'])
    err = np.abs(g['rgb'] - o['rgb']).max()
    print(f'{material}/{raster}: rgb max abs err {err:.3g}')
    assert err <= 1e-4
    cov = g['face_id'] >= 0
    assert cov.sum() > 1000 and g['rgb'][cov].std() > 0.01


def test_prefiltered_with_lamps_on_top(cuda, oracle_mod):
    sky = tina.Skybox(tina.procedural_sky(48, seed=5))
    light = tina.SkyboxLighting(sky, precision=4)
    light.add_light(pos=[2.0, 1.0, 3.0], color=[3.0, 3.0, 3.0])
    scene, _ = random_soup_scene(6, ntri=800, res=(96, 80), nlights=0, ibl=True, lighting=light, tonemap=False)
    g = _render(scene)
    o = oracle_mod.render(scene)
    assert np.array_equal(g['face_id'], o['face_id'])
    assert (np.abs(g['rgb'] - o['rgb']) / np.maximum(1.0, np.abs(o['rgb']))).max() <= 1e-4


def test_prefiltered_refuses_phong(cuda):
    sky = tina.Skybox(tina.procedural_sky(48, seed=1))
    scene, _ = random_soup_scene(6, ntri=50, res=(32, 32), material='classic', nlights=0, ibl=True,
                                 lighting=tina.SkyboxLighting(sky, precision=2))
    with pytest.raises(RuntimeError):
        scene.render()


def test_bake_sizes_follow_the_reference(cuda):
    sky = tina.Skybox(tina.procedural_sky(512, seed=0))
    t = tina.IBLTables(sky, precision=2)
    # resolution / 2**(4 step) per level, Lambert at resolution // 6 (material.py:295-300, :410)
    assert [m.shape[1] for m in t.spec] == [512, 471, 410, 310, 193, 84, 31]
    assert t.diffuse.shape[:2] == (170, 85)
    assert all(torch.isfinite(m.float()).all() for m in t.spec + [t.diffuse])
