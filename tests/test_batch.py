"""Batched multi-view rendering (t3_render_batch: two launches over every
view, direct work items or binned tiles) against per-scene Scene.render and
the oracle, plus the autotuner (its caching logic on the CPU, its choice on
the GPU)."""
import json

import numpy as np
import pytest

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N
from taichi_three_gb300.autotune import Autotuner


def test_autotuner_picks_fastest_and_persists(tmp_path):
    cost = {1: 5.0, 2: 1.0, 3: 3.0}
    calls = []
    clock = {'t': 0.0}

    def timer(fn):
        fn()
        return clock['t']

    def run(c):
        calls.append(c['k'])
        clock['t'] = cost[c['k']]

    path = str(tmp_path / 'tune.json')
    t = Autotuner(path=path, timer=timer)
    best, ms = t.tune(('w', 1), [dict(k=1), dict(k=2), dict(k=3)], run, repeats=2)
    assert best == dict(k=2) and ms == 1.0
    assert len(calls) == 9  # warm-up + 2 timed runs per candidate
    again = t.tune(('w', 1), [dict(k=1)], run)
    assert again == (dict(k=2), 1.0) and len(calls) == 9  # cached
    t2 = Autotuner(path=path, timer=timer)
    assert t2.tune(('w', 1), [dict(k=3)], run)[0] == dict(k=2)
    assert json.load(open(path))


def _small_batch(seed=0):
    scenes = tina.workloads.batch_scenes(6, seed=seed, t_min=200, t_max=30000,
                                         resolutions=(64, 96, 128, 200))
    # one scene with a face far larger than the CTA-cooperative threshold
    big = tina.Scene(256, 256, tonemap=True, smoothing=True)
    verts = np.array([[[-0.99, -0.99, 0.2], [0.99, -0.99, 0.2], [0, 0.99, 0.2]],
                      [[-0.5, -0.5, 0.5], [0.5, -0.5, 0.5], [0, 0.5, 0.5]]], np.float32)
    m = tina.SimpleMesh()
    m.set_face_verts(verts)
    m.set_face_norms(np.tile(np.array([0, 0, 1], np.float32), (2, 3, 1)))
    big.add_object(m, tina.Classic())
    scenes.append(big)
    return scenes


def _outputs(scene):
    import torch
    torch.cuda.synchronize()
    return (scene.img.cpu().numpy().copy(), scene.face_id.cpu().numpy().copy(),
            scene.engine.depth.cpu().numpy().copy(), scene.depth_f.cpu().numpy().copy())


BINNED = [dict(raster='binned', tile=t, tile_threads=th) for t, th in
          ((8, 64), (16, 128), (16, 256), (32, 128), (32, 256))]
CONFIGS = [dict(), dict(faces_per_item=256, pixels_per_item=1024, ctas_per_sm=1),
           dict(faces_per_item=4096, pixels_per_item=16384, ctas_per_sm=2)] + BINNED + [
           dict(raster='binned', tile=16, tile_threads=128, ctas_per_sm=1, bin_capacity=-2)]


@pytest.mark.gpu
@pytest.mark.parametrize('config', CONFIGS, ids=lambda c: '-'.join(f'{k}{v}' for k, v in c.items()) or 'default')
def test_batch_matches_single_renders(cuda, config):
    scenes = _small_batch()
    ref = []
    for s in scenes:
        s.render()
        ref.append(_outputs(s))
    b = tina.BatchRenderer(scenes, **config)
    b.render()
    assert b.status() == 0
    for s, (rgb, fid, dep, dpf) in zip(scenes, ref):
        g = _outputs(s)
        assert np.array_equal(g[1], fid)
        assert np.array_equal(g[2], dep)
        assert np.array_equal(g[3].view(np.uint32), dpf.view(np.uint32))
        assert np.abs(g[0] - rgb).max() <= 1e-5
    assert (ref[-1][1] == 0).sum() > 20000  # the big face covers most of its frame


@pytest.mark.gpu
def test_batch_binned_overflow_retries(cuda):
    # bins of 16 entries overflow on every view with more than a few faces per
    # tile; render() sees the status and renders again with larger bins
    scenes = _small_batch(3)
    ref = []
    for s in scenes:
        s.render()
        ref.append(_outputs(s))
    b = tina.BatchRenderer(scenes, raster='binned', tile=16, bin_capacity=16)
    b.render(check_bins=False)
    assert b.status() & N.T3_STATUS_BIN_OVERFLOW
    b.render()
    assert b.status() == 0 and b.last_config['bin_capacity'] < 0
    for s, (rgb, fid, dep, dpf) in zip(scenes, ref):
        g = _outputs(s)
        assert np.array_equal(g[1], fid)
        assert np.array_equal(g[2], dep)
        assert np.abs(g[0] - rgb).max() <= 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize('config', [dict(), dict(raster='binned', tile=32, tile_threads=256)],
                         ids=['direct', 'binned'])
def test_batch_against_oracle(cuda, oracle_mod, config):
    scenes = _small_batch(1)[:3]
    tina.BatchRenderer(scenes, **config).render()
    for s in scenes:
        g = _outputs(s)
        o = oracle_mod.render(s)
        assert np.array_equal(g[1], o['face_id'])
        assert np.array_equal(g[2], o['depth'])
        assert np.abs(g[0] - o['rgb']).max() <= 1e-4


@pytest.mark.gpu
def test_batch_autotune(cuda):
    scenes = _small_batch(2)
    b = tina.BatchRenderer(scenes)
    cands = [dict(faces_per_item=256, pixels_per_item=1024, ctas_per_sm=1),
             dict(faces_per_item=1024, pixels_per_item=4096, ctas_per_sm=2),
             dict(raster='binned', tile=16, tile_threads=128, bin_capacity=0),
             dict(raster='binned', tile=8, tile_threads=64, bin_capacity=4)]
    tuner = Autotuner()
    cfg, ms = b.autotune(candidates=cands, tuner=tuner)
    assert cfg in cands[:3] and ms > 0
    # the candidate whose 4-entry bins overflow is never timed
    assert [c for c, _ in tuner.log] == cands[:3]
    b.render()
    assert b.status() == 0


@pytest.mark.gpu
def test_tune_scene(cuda):
    scene, _ = tina.workloads.soup_scene(ntri=20000, res=(160, 120), seed=3)
    cfg, ms = tina.tune_scene(scene, tuner=Autotuner())
    assert cfg['raster'] in ('direct', 'binned') and ms > 0
    scene.render()
    assert scene.status() == 0
