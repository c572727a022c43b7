"""Generates tests/golden/postfx_golden.npz from the reference's own
post-processing passes (tina/postp/blooming.py Blooming.apply, tina/postp/fxaa.py
FXAA.apply), run under tests/golden/taichi_standin.py like make_golden.py.

Both passes read outside their fields at the image border (Blooming's final
bilerp, FXAA's neighbours and bilerp), which Taichi leaves undefined; the
stand-in's clamp_reads mode makes those reads take the nearest element, the
convention the CUDA passes and the oracle document.

Usage:  TINA_REFERENCE=/path/to/taichi_three python tests/golden/make_golden_postfx.py
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)


def inputs():
    """Seeded images: HDR ones for the bloom (about a fifth above the
    threshold 1, even and odd sizes) and a blocky one with hard colour edges
    for FXAA."""
    rng = np.random.Generator(np.random.PCG64(51))
    out = {}
    for name, (w, h) in (('bloom_even', (64, 48)), ('bloom_odd', (67, 45))):
        img = rng.uniform(0.0, 1.0, size=(w, h, 3))
        spots = rng.uniform(size=(w, h)) < 0.2
        img[spots] *= rng.uniform(2.0, 8.0, size=(int(spots.sum()), 1))
        out[name] = img.astype(np.float32)
    blocks = rng.uniform(0.0, 1.0, size=(8, 6, 3))
    img = np.repeat(np.repeat(blocks, 6, axis=0), 6, axis=1)[:46, :34]
    img = img + rng.normal(0, 0.01, size=img.shape)
    out['fxaa'] = np.clip(img, 0, 1).astype(np.float32)
    return out


def main():
    import make_golden
    make_golden.load_reference()
    import taichi_standin as ti
    blooming = importlib.import_module('tina.postp.blooming')
    fxaa = importlib.import_module('tina.postp.fxaa')
    ti.Field.clamp_reads = True
    arrays = inputs()
    out = {}
    for name, img in arrays.items():
        w, h = img.shape[:2]
        field = ti.Vector.field(3, float, (w, h))
        field.from_numpy(img)
        if name.startswith('bloom'):
            blooming.Blooming((w, h)).apply(field)
        else:
            fxaa.FXAA((w, h)).apply(field)
        out['out_' + name] = field.to_numpy().astype(np.float32)
        changed = int((np.abs(out['out_' + name] - img) > 1e-6).any(axis=-1).sum())
        print(f'{name}: {changed} of {w * h} pixels changed', flush=True)
    np.savez_compressed(os.path.join(HERE, 'postfx_golden.npz'),
                        **{'in_' + k: v for k, v in arrays.items()}, **out)


if __name__ == '__main__':
    main()
