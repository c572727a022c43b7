"""FramePipeline: a stream of frames with host inputs and host outputs, run on
scene replicas and streams, gives the images of one-at-a-time renders."""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina


def test_pipeline_needs_cuda_or_scenes():
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError):
            tina.FramePipeline([object()])
    else:
        with pytest.raises(ValueError):
            tina.FramePipeline([])


@pytest.mark.gpu
def test_pipeline_matches_serial_frames(cuda):
    nframes, ntri = 7, 3000
    frames = []
    for k in range(nframes):
        v, n, a = tina.workloads.soup_arrays(ntri, seed=100 + k, median_sigma=0.05)
        frames.append(tuple(torch.from_numpy(x).pin_memory() for x in (v, n, a)))
    # one replica per slot, plus a reference scene rendered one frame at a time
    built = [tina.workloads.soup_scene(ntri=ntri, res=(128, 96), seed=0, nlights=3) for _ in range(3)]
    ref_scene, ref_mesh = built[0]
    meshes = {id(s): m for s, m in built[1:]}

    def upload_to(m, k):
        v, n, a = frames[k]
        m.set_face_verts(v)
        m.set_face_norms(n)
        m.set_face_attrs(a)

    expected = []
    for k in range(nframes):
        upload_to(ref_mesh, k)
        ref_scene.render()
        expected.append(ref_scene.img.cpu().numpy().copy())
    pipe = tina.FramePipeline([s for s, _ in built[1:]])
    got = []
    for k in range(nframes):
        j = pipe.submit(lambda sc, k=k: upload_to(meshes[id(sc)], k))
        assert j == k
        if k >= 1:
            got.append(pipe.result(k - 1).numpy().copy())
    got.append(pipe.result(nframes - 1).numpy().copy())
    with pytest.raises(ValueError):
        pipe.result(0)  # its replica now holds a later frame
    for k in range(nframes):
        assert np.array_equal(got[k], expected[k]), k
    assert len({float(e.sum()) for e in expected}) == nframes  # the frames differ
