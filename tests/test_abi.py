"""CPU tests of the C ABI boundary and the host-side API logic (no GPU compute)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, 'include', 'tina3.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    return sorted(set(re.findall(r'^\s*int\s+(t3_\w+)\s*\(', src, flags=re.M)))


def test_library_exports_every_declared_entry_point():
    lib = N.load()
    names = header_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name
        assert name in N.SIGNATURES, f'{name} has no ctypes signature'


def test_struct_layouts_match():
    lib = N.load()
    N.check_layout(lib)
    n = lib.t3_struct_sizes(None, 0)
    assert n == len(N.STRUCTS)
    # lamps are read as float4 pairs: 16-byte aligned inside the scene
    assert (N.t3_scene.lighting.offset + N.t3_lighting.lights.offset) % 16 == 0
    assert C.sizeof(N.t3_light) % 16 == 0


def test_null_arguments_are_rejected_without_touching_the_device():
    lib = N.load()
    assert lib.t3_render(None, 0, 16, 0, None, 0, None, None, None) == N.T3_EINVAL
    assert lib.t3_clear(None, 10, None) == N.T3_EINVAL
    assert lib.t3_grid_normals(None, None, 4, 4, None) == N.T3_EINVAL
    assert lib.t3_tonemap(None, 3, None) == N.T3_EINVAL
    size = C.c_size_t()
    assert lib.t3_workspace_size(None, 0, 16, 0, C.byref(size)) == N.T3_EINVAL


def test_workspace_size_is_host_computable():
    lib = N.load()
    scene, mesh = tina.workloads.sphere_scene(64)
    sc, keep = scene.describe('cpu')
    size = C.c_size_t()
    assert lib.t3_workspace_size(C.byref(sc), N.T3_RASTER_DIRECT, 16, 0, C.byref(size)) == 0
    assert size.value >= 64 * 64 * 8 + 4 * mesh.get_nfaces()
    sc.frame.width = 0
    assert lib.t3_workspace_size(C.byref(sc), N.T3_RASTER_DIRECT, 16, 0, C.byref(size)) == N.T3_EINVAL


def test_pbr_compiles_to_expected_expression_table():
    mat, uses_attr = tina.compile_material(tina.PBR(basecolor=[0.8, 0.5, 0.2], metallic=0.3, roughness=0.4))
    ops = [mat.nodes[i].op for i in range(mat.nnodes)]
    assert not uses_attr
    assert mat.nodes[mat.root].op == N.T3_OP_MIX
    assert ops.count(N.T3_OP_FRESNEL) == 1  # f0 shared by Cook fresnel and the mix factor
    assert ops.count(N.T3_OP_LAMBERT) == 1 and ops.count(N.T3_OP_COOK) == 1
    fres = [i for i in range(mat.nnodes) if mat.nodes[i].op == N.T3_OP_FRESNEL][0]
    for ref in (mat.nodes[fres].a, mat.nodes[fres].b, mat.nodes[fres].c):
        assert ref < fres


def test_classic_int_shineness_is_flagged():
    mat, _ = tina.compile_material(tina.Classic())
    phong = [mat.nodes[i] for i in range(mat.nnodes) if mat.nodes[i].op == N.T3_OP_PHONG][0]
    m = mat.nodes[phong.a]
    assert m.op == N.T3_OP_CONST and m.c == 1 and m.v[0] == 32.0
    mat2, _ = tina.compile_material(tina.Phong())  # default 32.0 (float)
    phong2 = [mat2.nodes[i] for i in range(mat2.nnodes) if mat2.nodes[i].op == N.T3_OP_PHONG][0]
    assert mat2.nodes[phong2.a].c == 0


def test_node_coercion_and_errors():
    assert isinstance(tina.nodes.as_node(0.5), tina.Const)
    assert isinstance(tina.nodes.as_node('normal'), tina.Input)
    with pytest.raises(TypeError):
        tina.CookTorrance(roughness=0.2, bogus=1)
    with pytest.raises(ValueError):
        tina.Input('nope')
    with pytest.raises(NotImplementedError):
        tina.nodes.as_node('wood.png')


def test_facattr_material_requires_attributes():
    scene = tina.Scene(32)
    mesh = tina.SimpleMesh()
    mesh.set_face_verts(np.zeros((2, 3, 3), np.float32))
    scene.add_object(mesh, tina.workloads.pbr_face_material())
    with pytest.raises(ValueError):
        scene.describe('cpu')
    mesh.set_face_attrs(np.zeros((2, 5), np.float32))
    sc, keep = scene.describe('cpu')
    assert sc.objects[0].mesh.attr_stride == 5


def test_lighting_normalises_directions_and_marks_points():
    lt = tina.Lighting()
    lt.add_light(dir=[1, 2, 3], color=[0.9, 0.9, 0.9])
    lt.add_light(pos=[1, 1.5, 0.3], color=[1, 0, 0])
    d = np.array([1, 2, 3]) / np.sqrt(14)
    np.testing.assert_allclose(lt.light_dirs[0, :3], d.astype(np.float32))
    assert lt.light_dirs[0, 3] == 0 and lt.light_dirs[1, 3] == 1
    np.testing.assert_allclose(lt.light_dirs[1, :3], [1, 1.5, 0.3])
    lt.clear_lights()
    assert lt.nlights == 0


def test_engine_camera_matrices():
    e = tina.Engine(640, 480)
    view = tina.lookat(back=(0, 0, 3))
    proj = tina.perspective(60, 640 / 480)
    e.set_camera(view, proj)
    np.testing.assert_allclose(e.W2V, (proj @ view).astype(np.float32))
    np.testing.assert_allclose(e.V2W, np.linalg.inv(proj @ view).astype(np.float32), rtol=1e-6)
    # the camera sits at +3 z looking at the origin: the origin maps to NDC (0, 0)
    p = e.W2V @ np.array([0, 0, 0, 1.0])
    assert abs(p[0]) < 1e-7 and abs(p[1]) < 1e-7 and p[3] > 0


def test_matrix_helpers():
    np.testing.assert_allclose(tina.translate([1, 2, 3]) @ [0, 0, 0, 1], [1, 2, 3, 1])
    np.testing.assert_allclose(tina.scale(2) @ [1, 1, 1, 1], [2, 2, 2, 1])
    f = tina.frustum(-1, 1, -1, 1, 1, 100)
    assert f[3, 2] == -1 and f[3, 3] == 0
    q = tina.quaternion([0, 0, 0, 1])
    np.testing.assert_allclose(q, np.eye(4))


def test_sphere_face_count_matches_reference_generator():
    # Tina's PrimitiveMesh.sphere drops one triangle per pole quad
    assert tina.PrimitiveMesh.sphere(lons=64, lats=32).get_nfaces() == 64 * 32 * 2 - 2 * 64


def test_mesh_edit_flags_and_unsupported_nesting():
    base = tina.SimpleMesh()
    base.set_face_verts(np.zeros((3, 3, 3), np.float32))
    m = tina.MeshNoCulling(tina.MeshFlipNormal(tina.MeshTransform(base, tina.translate([1, 0, 0]))))
    desc = N.t3_mesh()
    m._t3_fill(desc, 'cpu', [])
    assert desc.flags == N.T3_MESH_TRANSFORM | N.T3_MESH_FLIP_NORMAL | N.T3_MESH_NOCULL
    assert m.get_nfaces() == 6
    bad = tina.MeshTransform(tina.MeshNoCulling(base))
    with pytest.raises(NotImplementedError):
        bad._t3_fill(N.t3_mesh(), 'cpu', [])


def test_unsupported_scene_options_raise():
    with pytest.raises(NotImplementedError):
        tina.Scene(64, ssao=True)
    with pytest.raises(ValueError):
        tina.Scene(64, raster='bogus')
