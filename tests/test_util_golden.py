"""The camera and transform helpers and the TAA running mean against golden
vectors from the reference's own tina/util/matrix.py and
tina/util/accumator.py (tests/golden/make_golden_util.py).  The matrices are
float64 numpy in both; the running mean is the oracle restatement that the
CUDA accumulation is held to by tests/test_postfx.py."""
import os
import sys

import numpy as np
import pytest

import taichi_three_gb300 as tina
from oracle import postfx_oracle as PF

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
sys.path.insert(0, GOLDEN)
import make_golden_util as recipe  # noqa: E402


@pytest.mark.parametrize('k', range(len(recipe.MATRIX_CALLS)))
def test_matrix_helpers_match_reference(k):
    fn, args, kwargs = recipe.MATRIX_CALLS[k]
    gold = np.load(os.path.join(GOLDEN, 'util_golden.npz'))[f'matrix_{k}']
    got = np.asarray(getattr(tina, fn)(*args, **kwargs), np.float64)
    np.testing.assert_allclose(got, gold, rtol=1e-12, atol=1e-12, err_msg=fn)


def test_taa_running_mean_matches_reference():
    d = np.load(os.path.join(GOLDEN, 'util_golden.npz'))
    src = d['in_frames']
    acc = np.zeros_like(src[0])
    for k in range(len(src)):
        acc = PF.accumulate(acc, src[k], k + 1)
        assert np.abs(acc - d[f'taa_{k}']).max() <= 1e-6, k
