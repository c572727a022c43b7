"""t3_render_noalloc: one frame with no device allocation by the library.

Some callers cannot allocate device memory: a renderer running inside a host
application that owns the GPU's memory and only hands over its input and
output buffers (a plug-in or frame callback where cudaMalloc is forbidden or
could stall).  For them t3_render_noalloc renders a frame with its scratch in a
fixed array built into libtina3.so.  This test calls it through the C ABI on
two different scenes in a row and checks each frame against t3_render (the
entry point with a caller-allocated workspace): face id, depth and float depth
bit-exact, scene.img within the 1e-4 tolerance the parity tests use.  It lives
in its own file that pytest collects last, and passes alone or after the rest.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-4


def _scenes():
    verts, norms, attrs = tina.workloads.soup_arrays(5000, seed=21, median_sigma=0.05)
    a, _ = tina.workloads.soup_scene(ntri=5000, res=(320, 200), seed=21, nlights=5,
                                     arrays=(verts, norms, attrs))
    b, _ = tina.workloads.sphere_scene(256)
    b.lighting.add_light(pos=[1.0, 2.0, 2.5], color=[2.0, 1.5, 1.0])
    return [a, b]


def _outputs(W, H, dev):
    return {'rgb': torch.full((W, H, 3), -7.0, device=dev),
            'face_id': torch.full((W, H), -7, dtype=torch.int32, device=dev),
            'depth': torch.full((W, H), -7, dtype=torch.int32, device=dev),
            'depth_f': torch.full((W, H), -7.0, device=dev)}


def test_noalloc_render_matches_t3_render_on_two_calls(cuda):
    lib = N.load()
    dev = cuda
    scenes = _scenes()
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    outs_all = [_outputs(*s.res, dev) for s in scenes]
    descs = []
    for s in scenes:
        for obj in s.objects:
            obj.pre_compute()
        descs.append(s.describe(dev))
    # two no-alloc frames back to back (the second reuses the scratch the first left)
    for (sc, _keep), o in zip(descs, outs_all):
        outs = N.t3_outputs(o['rgb'].data_ptr(), o['face_id'].data_ptr(), o['depth'].data_ptr(),
                            o['depth_f'].data_ptr())
        rc = lib.t3_render_noalloc(C.byref(sc), status.data_ptr(), C.byref(outs), stream)
        assert rc == N.T3_OK
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    # the same frames through t3_render with its allocated workspace
    for s, o in zip(scenes, outs_all):
        s.render()
        torch.cuda.synchronize()
        assert np.array_equal(o['face_id'].cpu().numpy(), s.face_id.cpu().numpy())
        assert np.array_equal(o['depth'].cpu().numpy(), s.engine.depth.cpu().numpy())
        assert np.array_equal(o['depth_f'].cpu().numpy().view(np.uint32),
                              s.depth_f.cpu().numpy().view(np.uint32))
        err = np.abs(o['rgb'].cpu().numpy() - s.img.cpu().numpy()).max()
        assert err <= RGB_TOL, err
        assert (o['face_id'] >= 0).sum().item() > 1000


def test_noalloc_rejects_frames_beyond_its_scratch(cuda):
    lib = N.load()
    scene, _ = tina.workloads.sphere_scene(64)
    sc, keep = scene.describe(cuda)
    sc.frame.width, sc.frame.height = 2048, 2048  # 4 Mpx > T3_NOALLOC_MAX_PIXELS
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    img = torch.empty(4, device=cuda)
    outs = N.t3_outputs(img.data_ptr(), None, None, None)
    rc = lib.t3_render_noalloc(C.byref(sc), status.data_ptr(), C.byref(outs),
                               torch.cuda.current_stream().cuda_stream)
    assert rc == N.T3_ETOOBIG
