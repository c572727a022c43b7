"""The oracle's sky background against golden vectors from the reference's own
background pass (tests/golden/make_golden_sky.py: Engine.render_background
with BackgroundShader over Skybox.sample, run under the Taichi stand-in): the
environment along every pixel's view ray, spheremap + bilerp of a seeded
32x16 HDR map, for two cameras.  Bar: within 1e-5 relative (the spherical
mapping's atan2 / acos differ by an ulp between libraries).  The CUDA
background is held to the oracle by tests/test_ibl.py."""
import os
import sys

import numpy as np
import pytest

import taichi_three_gb300 as tina

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
sys.path.insert(0, GOLDEN)
import make_golden_sky as recipe  # noqa: E402


@pytest.mark.parametrize('name', list(recipe.CAMERAS))
def test_sky_background_matches_reference(oracle_mod, name):
    d = np.load(os.path.join(GOLDEN, 'sky_golden.npz'))
    cam = recipe.CAMERAS[name]
    W, H = recipe.RES
    light = tina.SkyboxLighting(tina.Skybox(d['in_env'], half=False), mode='mc', spp=1)
    scene = tina.Scene(W, H, ibl=True, lighting=light, tonemap=False)
    scene.engine.set_camera(tina.lookat(back=cam['back']), tina.perspective(cam['fov'], W / H))
    gold = d['out_' + name]
    got = oracle_mod.render(scene)['rgb']
    assert (np.abs(got - gold) / np.maximum(1.0, np.abs(gold))).max() <= 1e-5
    assert gold.std() > 0.1  # the view sweeps across the map's structure
