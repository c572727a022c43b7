"""Mesh updates from host tensors: same-shape CPU float32 tensors are copied
into the existing device buffers (stream-ordered, asynchronous from pinned
memory), like Taichi's field.from_numpy; the frame matches the oracle."""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina

pytestmark = pytest.mark.gpu


def test_in_place_pinned_updates(cuda, oracle_mod):
    verts, norms, attrs = tina.workloads.soup_arrays(3000, 7, median_sigma=0.05, log_sd=0.5)
    scene, mesh = tina.workloads.soup_scene(ntri=3000, res=(96, 64), seed=7, arrays=(verts, norms, attrs))
    ptrs = (mesh.verts.data_ptr(), mesh.norms.data_ptr(), mesh.face_attr.data_ptr())
    v2 = torch.from_numpy(verts[::-1].copy()).pin_memory()
    n2 = torch.from_numpy(norms[::-1].copy()).pin_memory()
    a2 = torch.from_numpy(attrs[::-1].copy()).pin_memory()
    mesh.set_face_verts(v2)
    mesh.set_face_norms(n2)
    mesh.set_face_attrs(a2)
    assert (mesh.verts.data_ptr(), mesh.norms.data_ptr(), mesh.face_attr.data_ptr()) == ptrs
    scene.render()
    torch.cuda.synchronize()
    assert torch.equal(mesh.verts.cpu(), v2)
    o = oracle_mod.render(scene)
    assert np.array_equal(scene.face_id.cpu().numpy(), o['face_id'])
    assert np.abs(scene.img.cpu().numpy() - o['rgb']).max() <= 1e-4
    # a different face count reallocates
    mesh.set_face_verts(torch.from_numpy(verts[:100].copy()))
    assert mesh.get_nfaces() == 100 and mesh.verts.data_ptr() != ptrs[0]
