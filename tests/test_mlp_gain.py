"""What the learned IBL term gains over the method without it.

Workload: the 1080p soup (1M faces, per-face PBR) lit only by a seeded
procedural 1024 x 512 FP16 environment (sky gradient + 12 Gaussian lobes).
The network is trained here by the library's own kernels on 16M samples with
4096-sample Monte Carlo targets.  Against the FP64 oracle (4096 samples per
pixel, independent seed) on 4000 random covered pixels:
  * mean CIEDE2000 of the MLP frame < 1, and below that of 256-sample MC-IBL;
  * the MLP frame renders >= 3x faster than the 256-sample MC-IBL frame.
"""
import time

import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina

pytestmark = pytest.mark.gpu


def _frame_ms(scene, n):
    scene.render()
    torch.cuda.synchronize()
    times = []
    for _ in range(n):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        scene.render()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return float(np.median(times))


def test_mlp_ibl_beats_mc256(cuda, oracle_mod):
    sky = tina.Skybox(tina.procedural_sky(512, seed=0))
    t0 = time.time()
    net, losses = tina.train_for_skybox(sky, samples=1 << 24, spp=4096, steps=12000, batch=32768,
                                        log_every=2000)
    torch.cuda.synchronize()
    print(f'training: {time.time() - t0:.1f} s, loss {losses}')
    frames = {}
    for key, mode, spp in (('mlp', 'mlp', 1), ('mc256', 'mc', 256)):
        scene, _ = tina.workloads.ibl_soup_scene(skybox=sky, mode=mode, spp=spp, mlp=net)
        ms = _frame_ms(scene, 10 if mode == 'mlp' else 4)
        frames[key] = (ms, scene.img.cpu().numpy().reshape(-1, 3), scene)
    scene = frames['mlp'][2]
    fid = scene.face_id.cpu().numpy().ravel()
    cov = np.argwhere(fid >= 0).ravel()
    pick = np.sort(np.random.default_rng(0).choice(cov, 4000, replace=False))
    _, truth = oracle_mod.pixels_f64(scene, pick, spp=4096, seed=12345)
    de = {k: tina.colour.delta_e2000(v[1][pick], truth) for k, v in frames.items()}
    for k in frames:
        print(f'{k}: {frames[k][0]:.3f} ms/frame, mean dE2000 {de[k].mean():.3f}, '
              f'p95 {np.quantile(de[k], 0.95):.3f}')
    speedup = frames['mc256'][0] / frames['mlp'][0]
    print(f'speed-up over MC-256: {speedup:.2f}x')
    assert de['mlp'].mean() < 1.0
    assert de['mlp'].mean() < de['mc256'].mean()
    assert speedup >= 3.0
