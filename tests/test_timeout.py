"""The device-side timeout path (failure detection without a GPU fault).

Every wait of the library's kernels on an asynchronous copy or tensor-core
operation is bounded; when one runs out, the kernel records
T3_STATUS_TIMEOUT in the caller's status word, lets whatever it issued land,
and returns, so the context stays usable.  Here the binned tiles are made to
wait on a bin copy that is never issued (T3_STARVE_BIN_COPY) with a short
first-wait limit: every tile must give up, write background, and report the
timeout, and the next normal frame through the same workspace must match the
oracle bit for bit.  The learned-IBL network pass is starved the same way
(T3_STARVE_NETWORK).
"""
import ctypes as C

import numpy as np
import pytest
import torch

from helpers import random_soup_scene
from taichi_three_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _frame(lib, sc, ws, status, outs):
    N.check(lib.t3_render(C.byref(sc), N.T3_RASTER_BINNED, 16, 0, ws.data_ptr(), ws.numel(),
                          status.data_ptr(), C.byref(outs), torch.cuda.current_stream().cuda_stream),
            't3_render')
    torch.cuda.synchronize()
    return int(status.item())


def test_starved_bin_copy_times_out_then_next_frame_is_exact(cuda, oracle_mod):
    lib = N.load()
    scene, _ = random_soup_scene(3, ntri=3000, res=(128, 96), raster='binned', tile=16)
    for obj in scene.objects:
        obj.pre_compute()
    sc, keep = scene.describe(cuda)
    size = C.c_size_t()
    N.check(lib.t3_workspace_size(C.byref(sc), N.T3_RASTER_BINNED, 16, 0, C.byref(size)), 'size')
    ws = N.new_workspace(size.value, cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    W, H = scene.res
    rgb = torch.full((W, H, 3), -1.0, device=cuda)
    fid = torch.full((W, H), -7, dtype=torch.int32, device=cuda)
    dep = torch.full((W, H), -7, dtype=torch.int32, device=cuda)
    outs = N.t3_outputs(rgb.data_ptr(), fid.data_ptr(), dep.data_ptr(), None)

    flags = sc.frame.flags
    sc.frame.flags = flags | N.T3_STARVE_BIN_COPY
    sc.frame.wait_limit = 64
    st = _frame(lib, sc, ws, status, outs)
    assert st & N.T3_STATUS_TIMEOUT
    assert (fid == -1).all() and (dep == 2**30).all()  # every tile gave up: background
    bg = rgb[0, 0].clone()
    assert torch.equal(rgb, bg.expand_as(rgb))

    sc.frame.flags = flags
    sc.frame.wait_limit = 0
    st = _frame(lib, sc, ws, status, outs)
    assert st == 0
    o = oracle_mod.render(scene)
    assert np.array_equal(fid.cpu().numpy(), o['face_id'])
    assert np.array_equal(dep.cpu().numpy(), o['depth'])
    assert np.abs(rgb.cpu().numpy() - o['rgb']).max() <= 1e-4
    assert (o['face_id'] >= 0).sum() > 1000
    del keep


@pytest.mark.parametrize('entry', ['render', 'noalloc'])
def test_starved_network_times_out_then_next_frame_is_exact(cuda, entry):
    """The learned-IBL network pass made to wait on tensor-core work that is
    never issued (T3_STARVE_NETWORK): every wait gives up after wait_limit
    polls, the status reports the timeout, the covered pixels get no network
    colour, and the next normal frame repeats the first one bit for bit --
    through t3_render (row prepass + network kernel) and t3_render_noalloc
    (the one-kernel pass)."""
    import taichi_three_gb300 as tina
    sky = tina.Skybox(tina.procedural_sky(32, seed=5))
    light = tina.SkyboxLighting(sky, mode='mlp', mlp=tina.IBLNet(seed=1))
    scene, _ = tina.workloads.soup_scene(ntri=3000, res=(160, 120), seed=4, nlights=0, ibl=True,
                                         lighting=light,
                                         arrays=tina.workloads.soup_arrays(3000, 4, median_sigma=0.05))
    lib = N.load()
    for obj in scene.objects:
        obj.pre_compute()
    sc, keep = scene.describe(cuda)
    size = C.c_size_t()
    N.check(lib.t3_workspace_size(C.byref(sc), N.T3_RASTER_DIRECT, 16, 0, C.byref(size)), 'size')
    ws = N.new_workspace(size.value, cuda)
    status = torch.zeros(1, dtype=torch.int32, device=cuda)
    W, H = scene.res
    rgb = torch.full((W, H, 3), -7.0, device=cuda)
    fid = torch.full((W, H), -7, dtype=torch.int32, device=cuda)
    outs = N.t3_outputs(rgb.data_ptr(), fid.data_ptr(), None, None)
    stream = torch.cuda.current_stream().cuda_stream

    def frame():
        if entry == 'render':
            rc = lib.t3_render(C.byref(sc), N.T3_RASTER_DIRECT, 16, 0, ws.data_ptr(), ws.numel(),
                               status.data_ptr(), C.byref(outs), stream)
        else:
            rc = lib.t3_render_noalloc(C.byref(sc), status.data_ptr(), C.byref(outs), stream)
        assert rc == N.T3_OK
        torch.cuda.synchronize()
        return int(status.item())

    assert frame() == 0
    ref = rgb.clone()
    covered = fid >= 0
    assert covered.sum() > 2000
    rgb.fill_(-7.0)
    flags = sc.frame.flags
    sc.frame.flags = flags | N.T3_STARVE_NETWORK
    sc.frame.wait_limit = 64
    assert frame() & N.T3_STATUS_TIMEOUT
    assert (rgb[covered] == -7.0).all()
    if entry == 'render':
        # the prepass wrote the sky; the one-kernel pass stops walking its pixels
        assert torch.equal(rgb[~covered], ref[~covered])

    sc.frame.flags = flags
    sc.frame.wait_limit = 0
    assert frame() == 0
    assert torch.equal(rgb, ref)
    del keep
