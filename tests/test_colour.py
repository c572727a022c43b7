"""CIEDE2000 (taichi_three_gb300.colour) checked by properties: identity,
symmetry, agreement with an independent scalar restatement of the published
formula, monotonicity along a lightness ramp, and the CIELAB white / black
points.  (The formula's published test-pair table is not used.)"""
import math

import numpy as np

from taichi_three_gb300 import colour


def _de2000_scalar(l1, l2):
    """Scalar restatement of CIEDE2000 (Sharma, Wu & Dalal 2005), written
    independently of the vectorised one (float math, explicit branches)."""
    L1, a1, b1 = l1
    L2, a2, b2 = l2
    cb = (math.sqrt(a1 * a1 + b1 * b1) + math.sqrt(a2 * a2 + b2 * b2)) / 2
    g = 0.5 * (1 - math.sqrt(cb ** 7 / (cb ** 7 + 25 ** 7)))
    ap1, ap2 = a1 * (1 + g), a2 * (1 + g)
    cp1, cp2 = math.sqrt(ap1 * ap1 + b1 * b1), math.sqrt(ap2 * ap2 + b2 * b2)

    def hue(b, ap):
        if b == 0 and ap == 0:
            return 0.0
        h = math.degrees(math.atan2(b, ap))
        return h + 360 if h < 0 else h

    hp1, hp2 = hue(b1, ap1), hue(b2, ap2)
    if cp1 * cp2 == 0:
        dhp = 0.0
    elif abs(hp2 - hp1) <= 180:
        dhp = hp2 - hp1
    elif hp2 - hp1 > 180:
        dhp = hp2 - hp1 - 360
    else:
        dhp = hp2 - hp1 + 360
    dLp, dCp = L2 - L1, cp2 - cp1
    dHp = 2 * math.sqrt(cp1 * cp2) * math.sin(math.radians(dhp / 2))
    lbp, cbp = (L1 + L2) / 2, (cp1 + cp2) / 2
    if cp1 * cp2 == 0:
        hbp = hp1 + hp2
    elif abs(hp1 - hp2) <= 180:
        hbp = (hp1 + hp2) / 2
    elif hp1 + hp2 < 360:
        hbp = (hp1 + hp2 + 360) / 2
    else:
        hbp = (hp1 + hp2 - 360) / 2
    t = (1 - 0.17 * math.cos(math.radians(hbp - 30)) + 0.24 * math.cos(math.radians(2 * hbp))
         + 0.32 * math.cos(math.radians(3 * hbp + 6)) - 0.20 * math.cos(math.radians(4 * hbp - 63)))
    dth = 30 * math.exp(-((hbp - 275) / 25) ** 2)
    rc = 2 * math.sqrt(cbp ** 7 / (cbp ** 7 + 25 ** 7))
    sl = 1 + 0.015 * (lbp - 50) ** 2 / math.sqrt(20 + (lbp - 50) ** 2)
    sc = 1 + 0.045 * cbp
    sh = 1 + 0.015 * cbp * t
    rt = -math.sin(math.radians(2 * dth)) * rc
    return math.sqrt((dLp / sl) ** 2 + (dCp / sc) ** 2 + (dHp / sh) ** 2 + rt * (dCp / sc) * (dHp / sh))


def _pairs(n, seed):
    rng = np.random.default_rng(seed)
    a = rng.uniform(0, 1, (n, 3))
    b = np.clip(a + rng.normal(0, 0.05, (n, 3)), 0, 1)
    b[: n // 4] = rng.uniform(0, 1, (n // 4, 3))  # some far-apart pairs
    return a, b


def test_identity_and_symmetry():
    a, b = _pairs(2000, 0)
    assert np.all(colour.delta_e2000(a, a) == 0)
    assert np.allclose(colour.delta_e2000(a, b), colour.delta_e2000(b, a), atol=1e-9)


def test_agrees_with_scalar_restatement():
    a, b = _pairs(500, 1)
    la, lb = colour.srgb_to_lab(a), colour.srgb_to_lab(b)
    vec = colour.delta_e2000_lab(la, lb)
    ref = np.array([_de2000_scalar(x, y) for x, y in zip(la, lb)])
    assert np.abs(vec - ref).max() < 1e-9


def test_grey_axis_and_hue_wrap_cases():
    # achromatic pairs (C' = 0 branches) and hue pairs straddling 0 / 360 degrees
    cases = [((50, 0, 0), (60, 0, 0)), ((50, 2, -1e-3), (50, 2, 1e-3)), ((50, 0, 0), (50, 3, 0)),
             ((40, -10, -1), (40, -10, 1)), ((70, 5, 0.5), (70, 5, -0.5))]
    for l1, l2 in cases:
        v = colour.delta_e2000_lab(np.array(l1, float), np.array(l2, float))
        assert abs(float(v) - _de2000_scalar(l1, l2)) < 1e-9


def test_monotone_on_lightness_ramp():
    g = np.linspace(0, 1, 65)
    ramp = np.stack([g, g, g], axis=1)
    d = colour.delta_e2000(np.repeat(ramp[:1], len(g), 0), ramp)
    assert np.all(np.diff(d) > 0)


def test_lab_white_and_black():
    lab = colour.srgb_to_lab(np.array([[1.0, 1.0, 1.0], [0.0, 0.0, 0.0]]))
    assert np.allclose(lab[0], [100, 0, 0], atol=1e-3)
    assert np.allclose(lab[1], [0, 0, 0], atol=1e-9)
