"""Generates tests/golden/ibl_golden.npz from the reference's own IBL code.

Runs, under the Taichi stand-in of make_golden.py:
  * material.sample_ibl(tab, idir, nrm) -- the per-pixel lookup behind
    SkyboxLighting.shade_color (tina/core/lighting.py:20-21) -- of
    CookTorrance (tina/matr/material.py:256-277), Lambert (:441-442), a Mix of
    both (:141-145) and Scale (:187-191), on seeded maps and a seeded LUT that
    stand in for the baked tables (the lookup is pinned given its tables);
  * the samplers CookTorrance.sample (:365-384), Lambert.sample (:399-405),
    Phong.sample (:459-472) and MixMaterial.sample (:124-138) with fixed
    uniforms fed through the `rng` argument.
Inputs and outputs are saved together; tests/test_ibl_golden.py holds the
oracle's restatement to them.

Usage:  TINA_REFERENCE=/path/to/taichi_three python tests/golden/make_golden_ibl.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

ENV_RES = 48
N_DIRS = 64
ROUGH = [0.0, 0.01, 0.02, 0.045, 0.06, 0.1, 0.15, 0.2, 0.3, 0.42, 0.5, 0.6, 0.7, 0.85, 0.95, 1.0, 1.2]


def smooth_map(w, h, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    i, j = np.meshgrid(np.arange(w), np.arange(h), indexing='ij')
    ph = rng.uniform(0, 6.28, 3)
    base = 0.6 + 0.4 * np.stack([np.sin(i / 4.0 + ph[0]), np.cos(j / 3.0 + ph[1]),
                                 np.sin((i + j) / 5.0 + ph[2])], -1)
    return (base * rng.uniform(0.5, 1.5, size=(w, h, 3))).astype(np.float32)


def level_shapes():
    """The reference's map sizes for an environment of ENV_RES (material.py:295-300)."""
    levels = [0.03, 0.08, 0.18, 0.35, 0.65, 1.0]
    pairs = [(a, a - b) for a, b in zip(levels, [0] + levels)]
    res, shapes = ENV_RES, []
    for _, step in pairs:
        res = int(res / 2 ** (step * 4))
        shapes.append((2 * res, res))
    return shapes


def inputs():
    rng = np.random.Generator(np.random.PCG64(5))
    maps = [smooth_map(2 * ENV_RES, ENV_RES, 10)] + [smooth_map(w, h, 11 + k)
                                                     for k, (w, h) in enumerate(level_shapes())]
    diff = smooth_map(2 * (ENV_RES // 6), ENV_RES // 6, 30)
    lut = rng.uniform(0.0, 1.0, size=(3, 3, 3)).astype(np.float32)
    nrm = rng.normal(size=(N_DIRS, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    idir = rng.normal(size=(N_DIRS, 3))
    idir /= np.linalg.norm(idir, axis=1, keepdims=True)
    # mostly views from the front side of the normal, a few from behind
    flip = (np.sum(idir * nrm, axis=1) < 0) & (np.arange(N_DIRS) % 8 != 0)
    idir[flip] *= -1
    xi = rng.uniform(0.0, 1.0, size=(N_DIRS, 3)).astype(np.float32)
    f0 = rng.uniform(0.02, 0.9, size=(N_DIRS, 3)).astype(np.float32)
    fac = rng.uniform(0.0, 1.0, size=(N_DIRS, 3)).astype(np.float32)
    return {'maps': maps, 'diff': diff, 'lut': lut, 'nrm': nrm.astype(np.float32),
            'idir': idir.astype(np.float32), 'xi': xi, 'f0': f0, 'fac': fac}


class FixedRng:
    """The `rng` argument of material.sample(): the given uniforms in order."""

    def __init__(self, xs):
        self.xs = [np.float32(x) for x in xs]
        self.k = 0

    def random(self):
        x = self.xs[self.k]
        self.k += 1
        return x


def main():
    import make_golden
    tina, matrix = make_golden.load_reference()
    import importlib

    import taichi_standin as ti
    skybox = importlib.import_module('tina.skybox')
    advans = importlib.import_module('tina.advans')
    inp = inputs()

    def box(arr):
        b = skybox.Skybox(arr.shape[:2])
        b.img.from_numpy(arr)
        return b

    tab = {'spec': tuple(box(m) for m in inp['maps']), 'diff': box(inp['diff']),
           'lut': advans.texture_as_field(inp['lut'])}
    V = ti.Vector
    n = N_DIRS
    out = {'in_' + k: v for k, v in inp.items() if k != 'maps'}
    for k, m in enumerate(inp['maps']):
        out[f'in_map{k}'] = m
    out['in_rough'] = np.array(ROUGH, np.float32)

    def lookup(mat):
        res = np.zeros((n, 3), np.float32)

        @ti.kernel
        def run():
            for i in range(n):
                r = mat.sample_ibl(tab, V(list(inp['idir'][i])), V(list(inp['nrm'][i])))
                for c in range(3):
                    res[i, c] = r[c]
        run()
        return res

    # CookTorrance at every roughness (each with per-direction f0 through a Const)
    cook = np.zeros((len(ROUGH), n, 3), np.float32)
    for a, r in enumerate(ROUGH):
        for i in range(n):
            mat = tina.CookTorrance(roughness=float(r), fresnel=tuple(float(x) for x in inp['f0'][i]))
            cook[a, i] = lookup_one(ti, V, mat, tab, inp['idir'][i], inp['nrm'][i])
    out['out_cook'] = cook
    out['out_lambert'] = lookup(tina.Lambert())
    mix = tina.MixMaterial(tina.Lambert() * (0.7, 0.5, 0.3), tina.CookTorrance(roughness=0.27, fresnel=0.3),
                           0.35)
    out['out_mix'] = lookup(mix)
    out['out_scale'] = lookup(tina.Lambert() * 0.6)

    # samplers with fixed uniforms
    def sample(mat, xs):
        d, w = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
        for i in range(n):
            odir, wei, _ = run_sample(ti, V, mat, inp['idir'][i], inp['nrm'][i], xs[i])
            d[i] = as3(odir)
            w[i] = as3(wei)
        return d, w

    out['out_lambert_dir'], out['out_lambert_w'] = sample(tina.Lambert(), inp['xi'][:, :2])
    out['out_phong_dir'], out['out_phong_w'] = sample(tina.Phong(shineness=12.5), inp['xi'][:, :2])
    for r in (0.05, 0.4, 1.0):
        key = f'cook{int(r * 100):03d}'
        d = np.zeros((n, 3), np.float32)
        w = np.zeros((n, 3), np.float32)
        for i in range(n):
            mat = tina.CookTorrance(roughness=r, fresnel=tuple(float(x) for x in inp['f0'][i]))
            odir, wei, _ = run_sample(ti, V, mat, inp['idir'][i], inp['nrm'][i], inp['xi'][i, :2])
            d[i] = as3(odir)
            w[i] = as3(wei)
        out[f'out_{key}_dir'], out[f'out_{key}_w'] = d, w
    # MixMaterial: one choice draw, then the chosen child's two draws
    d = np.zeros((n, 3), np.float32)
    w = np.zeros((n, 3), np.float32)
    for i in range(n):
        mat = tina.MixMaterial(tina.Lambert(), tina.CookTorrance(roughness=0.4, fresnel=0.5),
                               tuple(float(x) for x in inp['fac'][i]))
        odir, wei, _ = run_sample(ti, V, mat, inp['idir'][i], inp['nrm'][i], inp['xi'][i])
        d[i] = as3(odir)
        w[i] = as3(wei)
    out['out_mix_dir'], out['out_mix_w'] = d, w
    np.savez_compressed(os.path.join(HERE, 'ibl_golden.npz'), **out)
    print('wrote', len(out), 'arrays')


def as3(x):
    """A vector, or a scalar broadcast (samplers return scalar weights)."""
    try:
        return [float(x[c]) for c in range(3)]
    except (TypeError, IndexError):
        return [float(x)] * 3


def lookup_one(ti, V, mat, tab, idir, nrm):
    box = {}

    @ti.kernel
    def run():
        box['r'] = mat.sample_ibl(tab, V(list(idir)), V(list(nrm)))
    run()
    return as3(box['r'])


def run_sample(ti, V, mat, idir, nrm, xs):
    box = {}
    rng = FixedRng(xs)

    @ti.kernel
    def run():
        box['r'] = mat.sample(V(list(idir)), V(list(nrm)), 1, rng)
    run()
    return box['r']


if __name__ == '__main__':
    main()
