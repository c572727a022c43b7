"""The oracle's image-based lighting held to the reference's own code
(tests/golden/ibl_golden.npz, made by tests/golden/make_golden_ibl.py, which
runs Tina's material.py under the Taichi stand-in):

* SkyboxLighting's prefiltered lookup, material.sample_ibl(tab, idir, nrm):
  CookTorrance at 17 roughness values across every level range and beyond
  1 (tina/matr/material.py:256-277), Lambert (:441-442), Mix (:141-145) and
  Scale (:187-191), on the same maps and LUT;
* the samplers with fixed uniforms: Lambert.sample (:399-405),
  CookTorrance.sample at three roughness values (:365-384), Phong.sample
  (:459-472) and MixMaterial.sample's choice and weights (:124-138).

Bar: float32 on both sides in the same operation order up to association,
1e-5 relative.  The CUDA kernels are held to the oracle on whole frames by
tests/test_ibl_prefiltered.py and tests/test_ibl.py.
"""
import os

import numpy as np
import pytest

import taichi_three_gb300 as tina
from taichi_three_gb300 import _native as N
from taichi_three_gb300.materials import compile_material

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'ibl_golden.npz'))
TOL = 1e-5


def close(a, b, tol=TOL):
    err = np.abs(a - b) / np.maximum(1.0, np.abs(b))
    assert err.max() <= tol, err.max()


def tables():
    keep = []
    T = N.t3_ibl_tables()
    for k in range(N.T3_IBL_LEVELS):
        m = np.ascontiguousarray(GOLD[f'in_map{k}'], np.float32)
        keep.append(m)
        T.spec[k].data = m.ctypes.data
        T.spec[k].w, T.spec[k].h = m.shape[:2]
        T.spec[k].half = 0
    d = np.ascontiguousarray(GOLD['in_diff'], np.float32)
    lut = np.ascontiguousarray(GOLD['in_lut'][..., :2], np.float32)
    keep += [d, lut]
    T.diffuse.data = d.ctypes.data
    T.diffuse.w, T.diffuse.h = d.shape[:2]
    T.lut = lut.ctypes.data
    T.lut_w, T.lut_h = lut.shape[:2]
    return T, keep


def lookup(oracle_mod, material, idir, nrm):
    T, keep = tables()
    mat, _ = compile_material(material, 0, 'cpu', keep)
    return oracle_mod.sample_ibl(mat, T, idir, nrm)


def test_cook_torrance_lookup_every_roughness(oracle_mod):
    idir, nrm, f0 = GOLD['in_idir'], GOLD['in_nrm'], GOLD['in_f0']
    for a, r in enumerate(GOLD['in_rough']):
        got = np.stack([lookup(oracle_mod, tina.CookTorrance(roughness=float(r), fresnel=tuple(f0[i].tolist())),
                               idir[i:i + 1], nrm[i:i + 1])[0] for i in range(len(idir))])
        close(got, GOLD['out_cook'][a])


def test_lambert_mix_scale_lookup(oracle_mod):
    idir, nrm = GOLD['in_idir'], GOLD['in_nrm']
    close(lookup(oracle_mod, tina.Lambert(), idir, nrm), GOLD['out_lambert'])
    mix = tina.MixMaterial(tina.Lambert() * (0.7, 0.5, 0.3), tina.CookTorrance(roughness=0.27, fresnel=0.3), 0.35)
    close(lookup(oracle_mod, mix, idir, nrm), GOLD['out_mix'])
    close(lookup(oracle_mod, tina.Lambert() * 0.6, idir, nrm), GOLD['out_scale'])
    assert np.abs(GOLD['out_mix'] - GOLD['out_lambert']).max() > 0.01  # the cases differ


@pytest.mark.parametrize('kind', ['lambert', 'phong', 'cook005', 'cook040', 'cook100'])
def test_leaf_samplers_with_fixed_uniforms(oracle_mod, kind):
    idir, nrm, xi, f0 = GOLD['in_idir'], GOLD['in_nrm'], GOLD['in_xi'][:, :2], GOLD['in_f0']
    n = len(idir)
    if kind == 'lambert':
        op, param = N.T3_OP_LAMBERT, np.zeros(n)
    elif kind == 'phong':
        op, param = N.T3_OP_PHONG, np.full(n, 12.5)
    else:
        op, param = N.T3_OP_COOK, np.full(n, int(kind[4:]) / 100.0)
    d, w = oracle_mod.sample_leaf(op, param, f0, idir, nrm, xi)
    close(d, GOLD[f'out_{kind}_dir'])
    close(w, GOLD[f'out_{kind}_w'])


def test_mix_sampler_choice_and_weight(oracle_mod):
    """MixMaterial(Lambert, CookTorrance(0.4, 0.5), fac).sample with uniforms
    (choice, u, v): the choice and its weight, then the chosen leaf's draw."""
    idir, nrm, xi, fac = GOLD['in_idir'], GOLD['in_nrm'], GOLD['in_xi'], GOLD['in_fac']
    n = len(idir)
    mw, second = oracle_mod.mix_choice(fac, xi[:, 0])
    ld, lw = oracle_mod.sample_leaf(N.T3_OP_LAMBERT, np.zeros(n), np.zeros((n, 3)), idir, nrm, xi[:, 1:])
    cd, cw = oracle_mod.sample_leaf(N.T3_OP_COOK, np.full(n, 0.4), np.full((n, 3), 0.5), idir, nrm, xi[:, 1:])
    d = np.where(second[:, None], cd, ld)
    w = np.where(second[:, None], cw, lw) * mw
    assert 0 < second.sum() < n
    close(d, GOLD['out_mix_dir'])
    close(w, GOLD['out_mix_w'])
