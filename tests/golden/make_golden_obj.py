"""Runs the reference's OBJ reader (tina/assimp/obj.py, numpy only: loaded
from its file without importing the tina package, which needs Taichi) on the
texts of obj_cases.py and stores the results in obj_golden.npz.

    python tests/golden/make_golden_obj.py /path/to/taichi_three
"""
import importlib.util
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from obj_cases import CASES  # noqa: E402


def main(ref_root):
    spec = importlib.util.spec_from_file_location('ref_obj', os.path.join(ref_root, 'tina', 'assimp', 'obj.py'))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = {}
    for name, text, kw in CASES:
        r = mod.readobj(io.BytesIO(text), **kw)
        for k in ('v', 'vt', 'vn', 'f'):
            out[f'{name}.{k}'] = np.asarray(r[k])
        if 'usemtl' in r:
            out[f'{name}.usemtl'] = np.array([f'{a}:{b.decode()}' for a, b in r['usemtl']])
    np.savez(os.path.join(HERE, 'obj_golden.npz'), **out)
    print('wrote', len(out), 'arrays')


if __name__ == '__main__':
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('TINA_REFERENCE')
    if not root:
        raise SystemExit('usage: make_golden_obj.py /path/to/taichi_three (or set TINA_REFERENCE)')
    main(root)
