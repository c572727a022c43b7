"""Fragment counting (t3_raster_fragments) against the oracle's own count of
pixel tests that pass (inside and below maxdepth), and the atomic-rate probe."""
import ctypes as C

import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N

pytestmark = pytest.mark.gpu


def test_fragment_count_is_plausible_and_stable(cuda):
    scene, _ = tina.workloads.soup_scene(ntri=20000, res=(160, 120), seed=2)
    scene.render()
    lib = N.load()
    sc, keep = scene.describe()
    counts = []
    for _ in range(2):
        n = C.c_int64()
        N.check(lib.t3_raster_fragments(C.byref(sc), scene._ws.data_ptr(), scene._ws.numel(), C.byref(n),
                                        torch.cuda.current_stream().cuda_stream), 'count')
        counts.append(n.value)
    covered = int((scene.face_id >= 0).sum())
    assert counts[0] == counts[1] and counts[0] >= covered > 0
    scene.render()  # the workspace is reusable afterwards
    assert int((scene.face_id >= 0).sum()) == covered


def test_red_min_probe(cuda):
    lib = N.load()
    buf = torch.full((1 << 16,), -1, dtype=torch.int64, device='cuda')
    N.check(lib.t3_red_min_rate(buf.data_ptr(), buf.numel(), 4, torch.cuda.current_stream().cuda_stream),
            'probe')
    got = buf.cpu().numpy().view(np.uint64)
    expect = (np.uint64(1) << np.uint64(32)) | np.arange(1 << 16, dtype=np.uint64)
    assert np.array_equal(got, expect)
