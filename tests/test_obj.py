"""OBJ reading (taichi_three_gb300.assimp.readobj) against the reference's own
reader run on the same texts (tests/golden/make_golden_obj.py ->
obj_golden.npz), and a MeshModel built from it rendered against the oracle."""
import io
import os
import sys

import numpy as np
import pytest

import taichi_three_gb300 as tina

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, 'golden'))
from obj_cases import CASES, CUBE  # noqa: E402

GOLD = np.load(os.path.join(HERE, 'golden', 'obj_golden.npz'))


@pytest.mark.parametrize('name,text,kw', CASES, ids=[c[0] for c in CASES])
def test_readobj_matches_reference(name, text, kw):
    r = tina.readobj(io.BytesIO(text), **kw)
    for k in ('v', 'vt', 'vn', 'f'):
        g = GOLD[f'{name}.{k}']
        assert r[k].shape == g.shape and r[k].dtype == g.dtype, (k, r[k].shape, g.shape)
        assert np.array_equal(r[k], g), k
    if f'{name}.usemtl' in GOLD:
        assert [f'{a}:{b.decode()}' for a, b in r['usemtl']] == GOLD[f'{name}.usemtl'].tolist()


def test_readobj_simple_and_path(tmp_path):
    p = tmp_path / 'cube.obj'
    p.write_bytes(CUBE)
    v, f = tina.readobj(str(p), simple=True)
    assert v.shape == (8, 3) and f.shape == (12, 3) and f.min() == 0 and f.max() == 7


@pytest.mark.gpu
def test_obj_model_render(cuda, oracle_mod):
    obj = tina.readobj(io.BytesIO(CUBE), scale=0.6)
    scene = tina.Scene(96, smoothing=True, texturing=True)
    scene.add_object(tina.MeshModel(obj), tina.Diffuse(color=tina.ChessboardTexture(size=0.25)))
    scene.engine.set_camera(tina.lookat(back=(1.5, 1.2, 2.5)), tina.perspective(60, 1))
    scene.render()
    o = oracle_mod.render(scene)
    assert np.array_equal(scene.face_id.cpu().numpy(), o['face_id'])
    assert (o['face_id'] >= 0).sum() > 1000
    assert np.abs(scene.img.cpu().numpy() - o['rgb']).max() <= 1e-4
