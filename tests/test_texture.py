"""Texturing (texturing=True): Texture (image, bilerp at texcoord * (shape - 1))
and ChessboardTexture nodes, evaluated by the shading kernels, against the
oracle (bit-exact id / depth, RGB within 1e-4)."""
import numpy as np
import pytest
import torch

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N
from taichi_three_gb300.materials import MaterialCompileError, compile_material


def _img(w, h, c, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(0, 1, (w, h, c) if c > 1 else (w, h)).astype(np.float32)


def test_compile_texture_nodes(cuda_or_cpu=None):
    tex = tina.Texture(_img(8, 4, 3, 0))
    m, _ = compile_material(tina.Diffuse(color=tex), device='cpu', keep=[])
    ops = [m.nodes[i].op for i in range(m.nnodes)]
    assert N.T3_OP_TEXTURE in ops
    k = ops.index(N.T3_OP_TEXTURE)
    assert m.nodes[m.nodes[k].a].op == N.T3_OP_INPUT and m.nodes[m.nodes[k].a].a == 3
    assert (m.textures[0].w, m.textures[0].h, m.textures[0].channels) == (8, 4, 3)
    c = tina.ChessboardTexture(size=0.25, color0=0.2, color1=(0.9, 0.5, 0.1))
    m, _ = compile_material(tina.Diffuse(color=c), device='cpu', keep=[])
    ops = [m.nodes[i].op for i in range(m.nnodes)]
    k = ops.index(N.T3_OP_CHECKER)
    assert m.nodes[int(m.nodes[k].v[0])].op == N.T3_OP_CONST
    many = tina.Diffuse(color=tina.Texture(_img(2, 2, 3, 1))) + tina.Diffuse(color=tina.Texture(_img(2, 2, 3, 2)))
    many = many + tina.Diffuse(color=tina.Texture(_img(2, 2, 3, 3)))
    many = many + tina.Diffuse(color=tina.Texture(_img(2, 2, 3, 4)))
    many = many + tina.Diffuse(color=tina.Texture(_img(2, 2, 3, 5)))
    with pytest.raises(MaterialCompileError):
        compile_material(many, device='cpu', keep=[])
    with pytest.raises(ValueError):
        tina.Texture(np.zeros((4, 4, 2), np.float32))
    with pytest.raises(NotImplementedError):
        tina.Texture('albedo.png')
    u8 = tina.Texture(np.full((2, 2, 3), 255, np.uint8))
    assert float(u8.data.max()) == 1.0


def _quad_scene(material, W=96, H=72):
    scene = tina.Scene(W, H, texturing=True, smoothing=True, tonemap=True)
    q = np.array([[-0.9, -0.8, 0.1], [0.8, -0.9, 0.2], [0.9, 0.85, 0.3], [-0.85, 0.9, 0.2]], np.float32)
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32)
    mesh = tina.SimpleMesh()
    mesh.set_face_verts(np.stack([q[[0, 1, 2]], q[[0, 2, 3]]]))
    mesh.set_face_norms(np.tile(np.array([0.1, 0.2, 1.0], np.float32), (2, 3, 1)))
    mesh.set_face_coors(np.stack([uv[[0, 1, 2]], uv[[0, 2, 3]]]))
    scene.add_object(mesh, material)
    scene.engine.set_camera(tina.lookat(back=(0, 0, 3)), tina.perspective(60, W / H))
    return scene


def _check(scene, oracle_mod):
    scene.render()
    torch.cuda.synchronize()
    o = oracle_mod.render(scene)
    assert np.array_equal(scene.face_id.cpu().numpy(), o['face_id'])
    assert np.array_equal(scene.engine.depth.cpu().numpy(), o['depth'])
    err = np.abs(scene.img.cpu().numpy() - o['rgb']).max()
    assert err <= 1e-4, err
    return o


@pytest.mark.gpu
@pytest.mark.parametrize('kind', ['rgb', 'scalar', 'checker', 'pbr'])
def test_texture_parity(cuda, oracle_mod, kind):
    if kind == 'rgb':
        mat = tina.Diffuse(color=tina.Texture(_img(13, 7, 3, 1)))
    elif kind == 'scalar':
        mat = tina.Lambert() * tina.Texture(_img(5, 9, 1, 2))
    elif kind == 'checker':
        mat = tina.Classic(color=tina.ChessboardTexture(size=0.125, color0=(0.9, 0.2, 0.1), color1=0.8))
    else:
        mat = tina.PBR(basecolor=tina.Texture(_img(16, 16, 3, 3)), metallic=tina.Texture(_img(4, 4, 1, 4)),
                       roughness=0.4)
    o = _check(_quad_scene(mat), oracle_mod)
    assert (o['face_id'] >= 0).sum() > 1000
    rgb = o['rgb'][o['face_id'] >= 0]
    assert rgb.std(axis=0).max() > 0.02  # the texture shows


@pytest.mark.gpu
def test_checker_on_sphere_binned(cuda, oracle_mod):
    scene = tina.Scene(128, texturing=True, smoothing=True, raster='binned')
    scene.add_object(tina.PrimitiveMesh.sphere(), tina.Diffuse(color=tina.ChessboardTexture(size=0.05)))
    scene.engine.set_camera(tina.lookat(back=(0, 0, 3)), tina.perspective(60, 1))
    _check(scene, oracle_mod)
