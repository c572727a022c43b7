"""Post-processing passes (Blooming, ToneMapping, FXAA, Accumator) on the GPU
against the numpy restatement in oracle/postfx_oracle.py, alone and chained by
Scene(blooming=True, fxaa=True, taa=True) in the reference's order."""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from oracle import postfx_oracle as PF

pytestmark = pytest.mark.gpu


def _hdr(W, H, seed):
    rng = np.random.default_rng(seed)
    img = np.exp(rng.normal(-0.5, 1.0, (W, H, 3))).astype(np.float32)
    img[W // 3: W // 2, H // 4: H // 2] *= 6.0  # a bright block with edges
    return img


@pytest.mark.parametrize('W,H', [(150, 96), (97, 64)])
def test_bloom(cuda, W, H):
    img = _hdr(W, H, 1)
    t = torch.from_numpy(img).cuda()
    tina.Blooming((W, H)).apply(t)
    ref = PF.bloom(img, radius=min(W, H) // 16)
    err = np.abs(t.cpu().numpy() - ref) / np.maximum(1.0, np.abs(ref))
    assert err.max() <= 1e-5, err.max()


def test_tonemap_exact(cuda, oracle_mod):
    img = _hdr(64, 48, 2)
    t = torch.from_numpy(img).cuda()
    tina.ToneMapping((64, 48)).apply(t)
    assert np.array_equal(t.cpu().numpy(), oracle_mod.aces(img))


def test_fxaa(cuda, oracle_mod):
    img = oracle_mod.aces(_hdr(120, 90, 3))
    t = torch.from_numpy(img).cuda()
    tina.FXAA((120, 90)).apply(t)
    ref = PF.fxaa(img)
    changed = np.abs(ref - img).max(axis=-1) > 0
    assert changed.sum() > 100  # edges were filtered
    assert np.abs(t.cpu().numpy() - ref).max() <= 1e-5


def test_scene_post_chain(cuda, oracle_mod):
    scene, _ = tina.workloads.soup_scene(ntri=4000, res=(128, 96), seed=5, blooming=True, fxaa=True)
    plain, _ = tina.workloads.soup_scene(ntri=4000, res=(128, 96), seed=5, tonemap=False)
    scene.render()
    plain.render()
    torch.cuda.synchronize()
    hdr = plain.img.cpu().numpy()
    o = oracle_mod.render(plain)
    assert np.array_equal(plain.face_id.cpu().numpy(), o['face_id'])
    ref = PF.fxaa(oracle_mod.aces(PF.bloom(hdr, radius=96 // 16)))
    got = scene.img.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-4


def test_taa_accumulates(cuda):
    scene, _ = tina.workloads.soup_scene(ntri=2000, res=(64, 48), seed=6, taa=True)
    frames = []
    for _ in range(4):
        scene.render()
        frames.append(scene.image.cpu().numpy().copy())
    acc = np.zeros_like(frames[0])
    for k, f in enumerate(frames, 1):
        acc = PF.accumulate(acc, f, k)
    assert np.abs(scene.img.cpu().numpy() - acc).max() <= 1e-6
    assert np.abs(frames[0] - frames[1]).max() > 0  # the pixel offsets differ between frames
    scene.clear()
    scene.render()
    assert np.array_equal(scene.img.cpu().numpy(), scene.image.cpu().numpy())
