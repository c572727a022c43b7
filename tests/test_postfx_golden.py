"""The post-processing restatement (oracle/postfx_oracle.py) against golden
vectors from the reference's own passes: tests/golden/make_golden_postfx.py
runs tina/postp/blooming.py Blooming.apply and tina/postp/fxaa.py FXAA.apply
under the Taichi stand-in on seeded images, with reads outside a field taking
the nearest element (Taichi leaves them undefined; the CUDA passes and the
oracle clamp).  The GPU passes are held to the same restatement by
tests/test_postfx.py."""
import os

import numpy as np
import pytest

from oracle import postfx_oracle as PF

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'postfx_golden.npz')


@pytest.mark.parametrize('name', ['bloom_even', 'bloom_odd'])
def test_bloom_matches_reference(name):
    d = np.load(GOLDEN)
    img, gold = d['in_' + name], d['out_' + name]
    assert (img > 1.0).any(axis=-1).mean() > 0.15  # enough pixels above the threshold
    got = PF.bloom(img)
    assert np.abs(got - gold).max() <= 1e-6 * max(1.0, float(np.abs(gold).max()))
    assert np.abs(gold - img).max() > 0.1  # the pass does something


def test_fxaa_matches_reference():
    d = np.load(GOLDEN)
    img, gold = d['in_fxaa'], d['out_fxaa']
    got = PF.fxaa(img)
    assert np.abs(got - gold).max() <= 1e-6
    assert (np.abs(gold - img) > 1e-3).any(axis=-1).sum() > 100  # edges were filtered
