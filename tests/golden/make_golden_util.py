"""Generates tests/golden/util_golden.npz from two small reference modules:
tina/util/matrix.py (the camera and transform helpers: lookat, ortho,
frustum, orthogonal, perspective, scale, translate, quaternion, eularXYZ,
evaluated on fixed arguments) and tina/util/accumator.py (Accumator.update,
the TAA running mean, over three seeded frames under the Taichi stand-in).

Usage:  TINA_REFERENCE=/path/to/taichi_three python tests/golden/make_golden_util.py
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

# (function name, positional args, keyword args): the same calls are made on
# taichi_three_gb300 by tests/test_util_golden.py
MATRIX_CALLS = [
    ('lookat', (), {}),
    ('lookat', ((0.2, -0.1, 0.3),), dict(back=(1.0, 2.0, 2.5))),
    ('lookat', (), dict(back=(0.0, -3.0, 0.5), up=(0.0, 0.0, 1.0))),
    ('ortho', (), {}),
    ('ortho', (-2.0, 1.5, -0.5, 3.0, 0.1, 20.0), {}),
    ('frustum', (), {}),
    ('frustum', (-0.3, 0.2, -0.1, 0.25, 0.5, 40.0), {}),
    ('orthogonal', (2.0, 1.6, -5.0, 5.0), {}),
    ('perspective', (), {}),
    ('perspective', (75.0, 16 / 9, 0.1, 100.0), {}),
    ('scale', (2.5,), {}),
    ('scale', ([0.5, 2.0, -1.0],), {}),
    ('translate', ([0.3, -0.7, 1.1],), {}),
    ('quaternion', ([0.1, 0.2, 0.3, 0.9273618495495703],), {}),
    ('eularXYZ', ([0.3, -0.5, 1.2],), {}),
]


def frames():
    rng = np.random.Generator(np.random.PCG64(91))
    return rng.uniform(0.0, 2.0, size=(3, 12, 9, 3)).astype(np.float32)


def main():
    import make_golden
    tina, matrix = make_golden.load_reference()
    import taichi_standin as ti
    accumator = importlib.import_module('tina.util.accumator')
    out = {}
    for k, (fn, args, kwargs) in enumerate(MATRIX_CALLS):
        out[f'matrix_{k}'] = np.asarray(getattr(matrix, fn)(*args, **kwargs), np.float64)
    src = frames()
    acc = accumator.Accumator(src.shape[1:3])
    field = ti.Vector.field(3, float, src.shape[1:3])
    for k in range(len(src)):
        field.from_numpy(src[k])
        acc.update(field)
        out[f'taa_{k}'] = acc.img.to_numpy().astype(np.float32)
    out['in_frames'] = src
    np.savez_compressed(os.path.join(HERE, 'util_golden.npz'), **out)
    print(f'{len(MATRIX_CALLS)} matrix calls, {len(src)} accumulated frames')


if __name__ == '__main__':
    main()
