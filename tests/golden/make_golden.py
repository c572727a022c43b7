"""Generates the golden fixtures tests/golden/*.npz from the reference itself.

Runs Tina's own source (the `tina` package of taichi-dev/taichi_three, read
from REFERENCE below) with tests/golden/taichi_standin.py installed as
`taichi`, renders every scene of recipes.py through the reference's Scene API,
and saves the input arrays plus the reference's outputs (scene.img,
engine.depth and the raster's occup buffer).  Only the subset of the package on
the raster path is imported: its subpackage __init__ files (which pull in the
path tracer, GUI and asset loaders) are replaced by empty packages, and
tina/hacker.py -- monkey-patches of Taichi internals -- by an empty module.

Usage:  TINA_REFERENCE=/path/to/taichi_three python tests/golden/make_golden.py [name ...]
"""
import importlib
import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# the taichi_three checkout to run (required: no default location is assumed)
REFERENCE = os.environ.get('TINA_REFERENCE')
sys.path.insert(0, HERE)

MODULES = ['tina.common', 'tina.advans', 'tina.matr.nodes', 'tina.matr.material', 'tina.core.engine',
           'tina.core.shader', 'tina.core.lighting', 'tina.core.triangle', 'tina.mesh.base',
           'tina.mesh.simple', 'tina.mesh.prim', 'tina.mesh.trans', 'tina.mesh.cull', 'tina.mesh.grid',
           'tina.mesh.norm', 'tina.mesh.conn', 'tina.mesh.model', 'tina.mesh.wire', 'tina.core.particle', 'tina.core.wireframe', 'tina.pars.simple', 'tina.postp.tonemap', 'tina.util.matrix', 'tina.scene.raster']


def load_reference():
    if not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, 'tina')):
        raise SystemExit('set TINA_REFERENCE to a taichi_three checkout (the directory holding tina/)')
    import taichi_standin
    sys.modules['taichi'] = taichi_standin
    sys.modules['taichi.lang'] = taichi_standin.lang
    root = os.path.join(REFERENCE, 'tina')
    pkg = types.ModuleType('tina')
    pkg.__path__ = [root]
    sys.modules['tina'] = pkg
    for sub in ('core', 'matr', 'mesh', 'pars', 'postp', 'scene', 'util'):
        m = types.ModuleType('tina.' + sub)
        m.__path__ = [os.path.join(root, sub)]
        sys.modules['tina.' + sub] = m
        setattr(pkg, sub, m)
    hacker = types.ModuleType('tina.hacker')
    hacker.__all__ = []
    sys.modules['tina.hacker'] = hacker
    # tina/util/matrix.py imports quaternion helpers it does not use on this path
    tr = types.ModuleType('transformations')
    for name in ('quaternion_matrix', 'quaternion_multiply', 'quaternion_from_matrix', 'euler_matrix'):
        setattr(tr, name, None)
    sys.modules['transformations'] = tr
    for name in MODULES:
        mod = importlib.import_module(name)
        for k, v in vars(mod).items():
            if not k.startswith('_') and not isinstance(v, types.ModuleType):
                setattr(pkg, k, v)
    return pkg, sys.modules['tina.util.matrix']


def main():
    from recipes import NAMES, build, inputs
    tina, matrix = load_reference()
    only = sys.argv[1:]
    for name in NAMES:
        if only and name not in only:
            continue
        t0 = time.time()
        arrays = inputs(name)
        scene, single = build(tina, name, arrays, matrix)
        scene.render()
        out = {'img': scene.img.to_numpy().astype(np.float32),
               'depth': scene.engine.depth.to_numpy().astype(np.int32)}
        if single:
            raster = getattr(scene, 'triangle_raster', None) or scene.particle_raster
            out['occup'] = raster.occup.to_numpy().astype(np.int32)
        np.savez_compressed(os.path.join(HERE, name + '.npz'),
                            **{'in_' + k: v for k, v in arrays.items()}, **out)
        cov = int((out['depth'] < 2**30).sum())
        print(f'{name}: {cov} covered pixels, {time.time() - t0:.1f} s', flush=True)


if __name__ == '__main__':
    main()
