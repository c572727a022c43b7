"""The lamp shading pass takes four consecutive pixels per thread: two 16-byte
key loads, and 16-byte background stores when all four are empty and the
output buffers are 16-byte aligned.  These tests hold the paths around that
against the oracle: frames whose pixel count is not a multiple of four (the
last quad is partly outside the frame), and outputs handed over through the C
ABI at addresses that are only 4-byte aligned (every quad falls back to
scalar stores).  Face id and depth bit-exact, RGB within 1e-4.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from helpers import random_soup_scene
from taichi_three_gb300 import _native as N

pytestmark = pytest.mark.gpu

RGB_TOL = 1e-4


def _assert_matches(g, o):
    assert np.array_equal(g['face_id'], o['face_id'])
    assert np.array_equal(g['depth'], o['depth'])
    assert np.array_equal(g['depth_f'].view(np.uint32), o['depth_f'].view(np.uint32))
    assert np.abs(g['rgb'] - o['rgb']).max() <= RGB_TOL


@pytest.mark.parametrize('res', [(97, 61), (33, 17), (1, 7), (5, 3)])
def test_frames_of_any_pixel_count(cuda, oracle_mod, res):
    scene, _ = random_soup_scene(31, ntri=800, res=res, nlights=3)
    scene.render()
    torch.cuda.synchronize()
    g = {'rgb': scene.img.cpu().numpy(), 'face_id': scene.face_id.cpu().numpy(),
         'depth': scene.engine.depth.cpu().numpy(), 'depth_f': scene.depth_f.cpu().numpy()}
    o = oracle_mod.render(scene)
    _assert_matches(g, o)
    if res[0] * res[1] > 100:
        assert (g['face_id'] >= 0).any() and (g['face_id'] < 0).any()


def test_outputs_at_unaligned_addresses(cuda, oracle_mod):
    W, H = 120, 90
    scene, _ = random_soup_scene(32, ntri=1500, res=(W, H), nlights=4)
    scene.render()  # the workspace and the reference outputs
    torch.cuda.synchronize()
    o = oracle_mod.render(scene)
    lib = N.load()
    n = W * H
    # one element past a 256-byte aligned start: 4-byte aligned only
    bufs = {'rgb': torch.full((3 * n + 1,), -7.0, device=cuda),
            'face_id': torch.full((n + 1,), -7, dtype=torch.int32, device=cuda),
            'depth': torch.full((n + 1,), -7, dtype=torch.int32, device=cuda),
            'depth_f': torch.full((n + 1,), -7.0, device=cuda)}
    outs = N.t3_outputs(bufs['rgb'][1:].data_ptr(), bufs['face_id'][1:].data_ptr(),
                        bufs['depth'][1:].data_ptr(), bufs['depth_f'][1:].data_ptr())
    assert all(p % 16 == 4 for p in (outs.rgb, outs.face_id, outs.depth, outs.depth_f))
    sc, keep = scene.describe(cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    ws = scene._ws  # the workspace scene.render() allocated
    for _ in range(2):  # the second frame starts from the keys the first one emptied
        rc = lib.t3_render(C.byref(sc), N.T3_RASTER_DIRECT, 16, 0, ws.data_ptr(), ws.numel(),
                           status.data_ptr(), C.byref(outs), torch.cuda.current_stream().cuda_stream)
        assert rc == N.T3_OK
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    g = {'rgb': bufs['rgb'][1:].view(W, H, 3).cpu().numpy(),
         'face_id': bufs['face_id'][1:].view(W, H).cpu().numpy(),
         'depth': bufs['depth'][1:].view(W, H).cpu().numpy(),
         'depth_f': bufs['depth_f'][1:].view(W, H).cpu().numpy()}
    _assert_matches(g, o)
    assert bufs['face_id'][0].item() == -7 and bufs['rgb'][0].item() == -7.0


def test_one_block_clear_when_the_hint_is_stale(cuda, oracle_mod):
    """The host remembers that a workspace's last direct frame emptied the keys
    and launches the next frame's clear as one block.  A CUDA graph captured
    then and replayed after a binned frame has scribbled over the workspace
    (and reset its key tag) must still give the oracle's frame: the one block
    finds the tag changed and clears every key."""
    W, H = 128, 96
    scene, _ = random_soup_scene(33, ntri=2000, res=(W, H), nlights=3)
    o = oracle_mod.render(scene)
    lib = N.load()
    sc, keep = scene.describe(cuda)
    sizes = []
    for mode in (N.T3_RASTER_DIRECT, N.T3_RASTER_BINNED):
        n = C.c_size_t()
        assert lib.t3_workspace_size(C.byref(sc), mode, 16, 0, C.byref(n)) == N.T3_OK
        sizes.append(n.value)
    ws = torch.zeros(max(sizes), dtype=torch.uint8, device=cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    bufs = {'rgb': torch.empty((W, H, 3), device=cuda), 'face_id': torch.empty((W, H), dtype=torch.int32, device=cuda),
            'depth': torch.empty((W, H), dtype=torch.int32, device=cuda), 'depth_f': torch.empty((W, H), device=cuda)}
    outs = N.t3_outputs(bufs['rgb'].data_ptr(), bufs['face_id'].data_ptr(), bufs['depth'].data_ptr(),
                        bufs['depth_f'].data_ptr())
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())

    def frame(mode, stream):
        rc = lib.t3_render(C.byref(sc), mode, 16, 0, ws.data_ptr(), ws.numel(), status.data_ptr(),
                           C.byref(outs), stream.cuda_stream)
        assert rc == N.T3_OK

    with torch.cuda.stream(side):
        frame(N.T3_RASTER_DIRECT, side)
        frame(N.T3_RASTER_DIRECT, side)  # the keys are now empty, and the host knows it
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=side):
            frame(N.T3_RASTER_DIRECT, side)  # captured with the one-block clear
    torch.cuda.synchronize()
    frame(N.T3_RASTER_BINNED, torch.cuda.current_stream())  # another layout over the same bytes
    torch.cuda.synchronize()
    for f in ('rgb', 'face_id', 'depth', 'depth_f'):
        bufs[f].fill_(-7)
    g.replay()
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    g_out = {k: v.cpu().numpy() for k, v in bufs.items()}
    _assert_matches(g_out, o)
