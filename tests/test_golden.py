"""Parity against golden vectors produced by the reference's own source.

tests/golden/*.npz were generated by tests/golden/make_golden.py, which runs
Tina's Python source (Scene, TriangleRaster, Shader, Lighting, materials, mesh
nodes, ToneMapping) under a pure-Python stand-in for the Taichi DSL.  Each
scene is rebuilt here with the same recipe (tests/golden/recipes.py) against
taichi_three_gb300, then rendered by the oracle (CPU) and by the CUDA library
(GPU).  Bar: raster outputs (occup / face id, int32 depth) bit-exact; scene.img
within 1e-5 absolute for the oracle, within the GPU bar of 1e-4 for the CUDA
path (relative for HDR scenes without tonemap).
"""
import os
import sys

import numpy as np
import pytest

import taichi_three_gb300 as tina

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
sys.path.insert(0, GOLDEN)
import recipes  # noqa: E402

IMG_TOL = 1e-5
GPU_TOL = 1e-4


def load(name):
    d = np.load(os.path.join(GOLDEN, name + '.npz'))
    arrays = {k[3:]: d[k] for k in d.files if k.startswith('in_')}
    gold = {k: d[k] for k in d.files if not k.startswith('in_')}
    return arrays, gold


def check(name, out, gold, scene, single, tol=IMG_TOL):
    assert np.array_equal(out['depth'], gold['depth']), f'{name}: depth differs'
    if single:
        assert np.array_equal(out['face_id'], gold['occup']), f'{name}: occup differs'
    diff = np.abs(out['rgb'] - gold['img'])
    if not scene.tonemap:
        diff = diff / np.maximum(1.0, np.abs(gold['img']))
    err = float(diff.max())
    assert err <= tol, f'{name}: img err {err}'
    return err


@pytest.mark.parametrize('name', recipes.NAMES)
def test_oracle_matches_reference_golden(oracle_mod, name):
    arrays, gold = load(name)
    scene, single = recipes.build(tina, name, arrays, tina)
    out = oracle_mod.render(scene)
    assert (gold['depth'] < 2**30).sum() > 100
    check(name, out, gold, scene, single)


@pytest.mark.gpu
@pytest.mark.parametrize('name', recipes.NAMES)
def test_cuda_matches_reference_golden(cuda, name):
    import torch
    arrays, gold = load(name)
    scene, single = recipes.build(tina, name, arrays, tina)
    scene.render()
    torch.cuda.synchronize()
    out = {'rgb': scene.img.cpu().numpy(), 'face_id': scene.face_id.cpu().numpy(),
           'depth': scene.engine.depth.cpu().numpy()}
    err = check(name, out, gold, scene, single, tol=GPU_TOL)
    print(f'{name}: img err {err:.3g}')
