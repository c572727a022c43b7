"""Known-answer tests of the oracle (CPU restatement of Tina's raster + shade).

The reference ships no golden images, so these pin the restatement to answers
derived by hand from the reference's formulas: coverage at exact pixel centres
with the inclusive edge test (tina/core/triangle.py:115-120), the lowest-id tie
rule of the serial `atomic_min(...) > depth` (triangle.py:123), back-face
culling (:95-98), the all-outside clip (:100-104), the depth quantisation
(:121-122), the lamp falloff (tina/core/lighting.py:84-98), the BRDFs
(tina/matr/material.py) and ACES (tina/advans.py:32-34).
"""
import numpy as np
import pytest

import taichi_three_gb300 as tina
from helpers import flat_scene, random_soup_scene

pytestmark = []


def coverage(out):
    return out['face_id'] >= 0


def test_single_triangle_pixel_centres(oracle_mod):
    # a=(0,0) b=(8,0) c=(0,8): pixel (i, j) is inside iff (i+.5)+(j+.5) <= 8
    scene, _ = flat_scene([[(0, 0), (8, 0), (0, 8)]])
    out = oracle_mod.render(scene)
    i, j = np.meshgrid(np.arange(8), np.arange(8), indexing='ij')
    expect = (i + j) <= 7
    assert np.array_equal(coverage(out), expect)
    assert expect.sum() == 36
    assert (out['face_id'][expect] == 0).all()


@pytest.mark.parametrize('order', [0, 1])
def test_shared_edge_tie_goes_to_lowest_id(oracle_mod, order):
    lower = [(0, 0), (8, 0), (0, 8)]
    upper = [(8, 0), (8, 8), (0, 8)]
    tris = [lower, upper] if order == 0 else [upper, lower]
    scene, _ = flat_scene(tris)
    out = oracle_mod.render(scene)
    i, j = np.meshgrid(np.arange(8), np.arange(8), indexing='ij')
    on_edge = (i + j) == 7
    assert coverage(out).all()
    # both faces cover the diagonal at equal depth: face 0 keeps it
    assert (out['face_id'][on_edge] == 0).all()
    lower_id = 0 if order == 0 else 1
    expect_lower = ((i + j) <= 7) & ~(on_edge & (lower_id != 0))
    assert np.array_equal(out['face_id'] == lower_id, expect_lower)


def test_backface_culling(oracle_mod):
    cw = [[(0, 0), (0, 8), (8, 0)]]
    out = oracle_mod.render(flat_scene(cw)[0])
    assert not coverage(out).any()
    out = oracle_mod.render(flat_scene(cw, culling=False)[0])
    assert coverage(out).sum() == 36


def test_clip_drops_faces_with_all_vertices_outside(oracle_mod):
    huge = [[(-20, -20), (40, -20), (-20, 40)]]
    assert not coverage(oracle_mod.render(flat_scene(huge)[0])).any()
    assert coverage(oracle_mod.render(flat_scene(huge, clipping=False)[0])).all()


def test_nearest_face_wins_regardless_of_order(oracle_mod):
    a = [(0, 0), (8, 0), (0, 8)]
    for z in ([0.6, 0.3], [0.3, 0.6]):
        out = oracle_mod.render(flat_scene([a, a], z=z)[0])
        near = int(np.argmin(z))
        assert (out['face_id'][coverage(out)] == near).all()
        d = out['depth'][coverage(out)]
        df = out['depth_f'][coverage(out)]
        assert np.all(np.abs(df - np.float32(0.3)) < 1e-7)
        assert np.array_equal(d, (df * np.float32(2**30)).astype(np.int32))


def test_empty_pixels_keep_maxdepth_and_background(oracle_mod):
    scene, _ = flat_scene([[(0, 0), (4, 0), (0, 4)]], bgcolor=0.25, tonemap=False)
    out = oracle_mod.render(scene)
    empty = ~coverage(out)
    assert empty.any()
    assert (out['depth'][empty] == 2**30).all()
    assert (out['face_id'][empty] == -1).all()
    assert np.all(out['rgb'][empty] == np.float32(0.25))


def test_point_light_inverse_square(oracle_mod):
    scene, _ = flat_scene([[(-8, -8), (24, -8), (-8, 24)]], W=16, H=16, clipping=False)
    scene.lighting.clear_lights()
    scene.lighting.set_ambient_light([0, 0, 0])
    lp = np.array([0.3, -0.2, 1.5])
    scene.lighting.add_light(pos=lp.tolist(), color=[2.0, 1.0, 0.5])
    out = oracle_mod.render(scene)
    for (x, y) in [(3, 4), (6, 6), (12, 2)]:
        p = np.array([(x + 0.5) / 16 * 2 - 1, (y + 0.5) / 16 * 2 - 1, -0.5])
        L = lp - p
        d = np.linalg.norm(L)
        cos = L[2] / d
        expect = cos * np.array([2.0, 1.0, 0.5]) / d**2 / np.pi
        np.testing.assert_allclose(out['rgb'][x, y], expect, rtol=2e-6)


def _pbr_expected(n, v, ldir, lcol, albedo, metallic, roughness, specular=0.5):
    """Independent float64 evaluation of PBR's lamp term (material.py:323-362, 701-706)."""
    f0 = metallic * albedo + (1 - metallic) * 0.16 * specular**2
    h = (ldir + v) / np.linalg.norm(ldir + v)
    NoH = max(1e-10, h @ n)
    NoL = max(1e-10, ldir @ n)
    NoV = max(1e-10, v @ n)
    VoH = min(1 - 1e-10, max(1e-10, h @ v))
    a2 = max(1e-6, roughness**2)
    D = a2 / (1 - NoH**2 * (1 - a2))**2
    k = a2 / 2
    G = 1 / (NoV * k + 1 - k) / (NoL * k + 1 - k) / ((1 - a2) + 4 * np.pi * a2)
    F = f0 + (1 - f0) * (1 - VoH)**5
    brdf = (1 - f0) * albedo / np.pi + f0 * F * G * D
    return (ldir @ n) * lcol * brdf


def test_pbr_lamp_term_matches_independent_formula(oracle_mod):
    albedo = np.array([0.8, 0.5, 0.2])
    for metallic, roughness in [(0.0, 0.4), (1.0, 0.15), (0.3, 0.8)]:
        scene, _ = flat_scene([[(-8, -8), (24, -8), (-8, 24)]], W=16, H=16, clipping=False,
                              material=tina.PBR(basecolor=albedo.tolist(), metallic=metallic,
                                                roughness=roughness))
        scene.lighting.clear_lights()
        scene.lighting.set_ambient_light([0, 0, 0])
        ldir = np.array([0.3, 0.4, 1.0])
        scene.lighting.add_light(dir=ldir.tolist(), color=[1.0, 0.9, 0.8])
        out = oracle_mod.render(scene)
        ldir = ldir / np.linalg.norm(ldir)
        n = np.array([0, 0, 1.0])
        v = np.array([0, 0, 1.0])
        expect = _pbr_expected(n, v, ldir, np.array([1.0, 0.9, 0.8]), albedo, metallic, roughness)
        np.testing.assert_allclose(out['rgb'][5, 7], expect, rtol=5e-5)


def test_classic_phong_term(oracle_mod):
    scene, _ = flat_scene([[(-8, -8), (24, -8), (-8, 24)]], W=16, H=16, clipping=False,
                          material=tina.Classic(color=0.7))
    scene.lighting.clear_lights()
    scene.lighting.set_ambient_light([0.05, 0.05, 0.05])
    ldir = np.array([0.1, 0.05, 1.0])
    scene.lighting.add_light(dir=ldir.tolist())
    out = oracle_mod.render(scene)
    ldir = ldir / np.linalg.norm(ldir)
    n = v = np.array([0, 0, 1.0])
    r = -ldir - 2 * (n @ -ldir) * n
    phong = max(0, v @ r)**32 * 34 / 2
    brdf = 0.6 * 0.7 / np.pi + 0.4 * phong
    amb = 0.05 * (0.6 * 0.7 + 0.4)
    np.testing.assert_allclose(out['rgb'][5, 7], amb + (ldir @ n) * brdf, rtol=5e-5)


def test_aces_fixed_points(oracle_mod):
    x = np.array([0.0, 1.0, 1e6], np.float32)
    y = oracle_mod.aces(x)
    assert y[0] == 0.0
    np.testing.assert_allclose(y[1], 2.54 / 3.16, rtol=1e-6)
    np.testing.assert_allclose(y[2], 2.51 / 2.43, rtol=1e-5)
    np.testing.assert_allclose(tina.aces_tonemap(1.0), 2.54 / 3.16)


@pytest.mark.parametrize('seed', [1, 2, 3])
def test_serial_and_parallel_modes_agree(oracle_mod, seed):
    scene, _ = random_soup_scene(seed, ntri=800)
    a = oracle_mod.render(scene, mode=0)
    b = oracle_mod.render(scene, mode=1)
    assert coverage(a).sum() > 100
    for k in ('face_id', 'depth', 'depth_f', 'rgb'):
        assert np.array_equal(a[k], b[k]), k


def test_fp64_twin_agrees_away_from_edges(oracle_mod):
    scene, _ = random_soup_scene(4, ntri=400)
    a = oracle_mod.render(scene)
    b = oracle_mod.render(scene, fp64=True)
    same = a['face_id'] == b['face_id']
    assert same.mean() > 0.97
    err = np.abs(a['rgb'][same] - b['rgb'][same])
    assert err.max() < 1e-4


def test_grid_normals_flat_and_tilted(oracle_mod):
    g = tina.MeshGrid(6)
    pos = g.pos.cpu().numpy()
    n = oracle_mod.grid_normals(pos)
    assert np.allclose(n, [0, 0, 1])
    pos2 = pos.copy()
    pos2[..., 2] = 0.5 * pos2[..., 0]
    n2 = oracle_mod.grid_normals(pos2)
    expect = np.array([-0.5, 0, 1]) / np.sqrt(1.25)
    assert np.allclose(n2, expect, atol=1e-6)


def test_multi_object_winner_and_shading(oracle_mod):
    # object 0 behind object 1 on the left half; serial per-object loop
    # (tina/scene/raster.py:183-187) equals the packed-key parallel result
    scene = tina.Scene(16, 16, tonemap=True, smoothing=False)
    m0 = tina.SimpleMesh()
    m0.set_face_verts(np.array([[[-1, -1, -0.7], [1, -1, -0.7], [-1, 1, -0.7]]], np.float32))
    m1 = tina.SimpleMesh()
    m1.set_face_verts(np.array([[[-1, -1, -0.2], [0.2, -1, -0.2], [-1, 0.2, -0.2]]], np.float32))
    scene.add_object(m0, tina.Diffuse(color=0.5))
    scene.add_object(m1, tina.Lamp(color=[1.0, 0.2, 0.1]))
    a = oracle_mod.render(scene, mode=0)
    b = oracle_mod.render(scene, mode=1)
    assert set(np.unique(a['face_id'])) == {-1, 0, 1}
    for k in ('face_id', 'depth', 'rgb'):
        assert np.array_equal(a[k], b[k]), k
    lamp = a['face_id'] == 1
    np.testing.assert_allclose(a['rgb'][lamp][0], tina.aces_tonemap(np.array([1.0, 0.2, 0.1])), rtol=1e-6)


@pytest.mark.parametrize('lighting', ['lamps', 'mc'])
def test_sampled_pixels_equal_the_whole_frame(oracle_mod, lighting):
    """oracle.pixels_f32 (the oracle of sampled pixels in frames too large to
    shade whole) returns the whole-frame render's own values bit for bit,
    Monte Carlo stream included."""
    opts = {}
    if lighting == 'mc':
        sky = tina.Skybox(tina.procedural_sky(16, seed=2))
        opts = dict(ibl=True, lighting=tina.SkyboxLighting(sky, mode='mc', spp=8, seed=7), nlights=0)
    scene, _ = random_soup_scene(9, ntri=500, res=(48, 40), **opts)
    full = oracle_mod.render(scene)
    rng = np.random.default_rng(0)
    px = rng.choice(48 * 40, 400, replace=False)
    rgb, fid = oracle_mod.pixels_f32(scene, px)
    assert np.array_equal(fid, full['face_id'].reshape(-1)[px])
    assert (fid >= 0).sum() > 50
    assert np.array_equal(rgb.view(np.uint32), full['rgb'].reshape(-1, 3)[px].view(np.uint32))
