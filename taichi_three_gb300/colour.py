"""Colour difference for image comparisons: CIEDE2000.

Images are compared as displayed: scene.img (post-ACES) is taken as
sRGB-encoded display values in [0, 1], decoded to linear RGB, converted to
CIE XYZ (D65) and CIELAB, and compared with the CIEDE2000 formula of Sharma,
Wu and Dalal, "The CIEDE2000 color-difference formula: implementation notes,
supplementary test data, and mathematical observations" (Color Research and
Application 30(1), 2005), with kL = kC = kH = 1.
"""
import numpy as np

# linear sRGB (D65) -> XYZ, IEC 61966-2-1
_RGB2XYZ = np.array([[0.4124564, 0.3575761, 0.1804375],
                     [0.2126729, 0.7151522, 0.0721750],
                     [0.0193339, 0.1191920, 0.9503041]])
_WHITE = np.array([0.95047, 1.0, 1.08883])


def srgb_to_linear(c):
    c = np.clip(np.asarray(c, np.float64), 0.0, 1.0)
    return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)


def srgb_to_lab(c):
    """Display sRGB [..., 3] -> CIELAB [..., 3] (D65 white)."""
    xyz = srgb_to_linear(c) @ _RGB2XYZ.T / _WHITE
    d = 6.0 / 29.0
    f = np.where(xyz > d ** 3, np.cbrt(xyz), xyz / (3 * d * d) + 4.0 / 29.0)
    L = 116.0 * f[..., 1] - 16.0
    a = 500.0 * (f[..., 0] - f[..., 1])
    b = 200.0 * (f[..., 1] - f[..., 2])
    return np.stack([L, a, b], axis=-1)


def delta_e2000_lab(lab1, lab2):
    """CIEDE2000 between CIELAB arrays [..., 3] (float64)."""
    lab1 = np.asarray(lab1, np.float64)
    lab2 = np.asarray(lab2, np.float64)
    L1, a1, b1 = lab1[..., 0], lab1[..., 1], lab1[..., 2]
    L2, a2, b2 = lab2[..., 0], lab2[..., 1], lab2[..., 2]
    c7 = 25.0 ** 7
    Cbar = 0.5 * (np.hypot(a1, b1) + np.hypot(a2, b2))
    G = 0.5 * (1.0 - np.sqrt(Cbar ** 7 / (Cbar ** 7 + c7)))
    a1p, a2p = (1.0 + G) * a1, (1.0 + G) * a2
    C1p, C2p = np.hypot(a1p, b1), np.hypot(a2p, b2)
    h1p = np.where((a1p == 0) & (b1 == 0), 0.0, np.degrees(np.arctan2(b1, a1p)) % 360.0)
    h2p = np.where((a2p == 0) & (b2 == 0), 0.0, np.degrees(np.arctan2(b2, a2p)) % 360.0)
    chroma0 = C1p * C2p == 0
    dh = h2p - h1p
    dh = np.where(dh > 180.0, dh - 360.0, np.where(dh < -180.0, dh + 360.0, dh))
    dh = np.where(chroma0, 0.0, dh)
    dL = L2 - L1
    dC = C2p - C1p
    dH = 2.0 * np.sqrt(C1p * C2p) * np.sin(np.radians(dh) / 2.0)
    Lbar = 0.5 * (L1 + L2)
    Cbarp = 0.5 * (C1p + C2p)
    hsum = h1p + h2p
    hbar = np.where(np.abs(h1p - h2p) <= 180.0, 0.5 * hsum,
                    np.where(hsum < 360.0, 0.5 * (hsum + 360.0), 0.5 * (hsum - 360.0)))
    hbar = np.where(chroma0, hsum, hbar)
    T = (1.0 - 0.17 * np.cos(np.radians(hbar - 30.0)) + 0.24 * np.cos(np.radians(2.0 * hbar))
         + 0.32 * np.cos(np.radians(3.0 * hbar + 6.0)) - 0.20 * np.cos(np.radians(4.0 * hbar - 63.0)))
    dtheta = 30.0 * np.exp(-(((hbar - 275.0) / 25.0) ** 2))
    RC = 2.0 * np.sqrt(Cbarp ** 7 / (Cbarp ** 7 + c7))
    SL = 1.0 + 0.015 * (Lbar - 50.0) ** 2 / np.sqrt(20.0 + (Lbar - 50.0) ** 2)
    SC = 1.0 + 0.045 * Cbarp
    SH = 1.0 + 0.015 * Cbarp * T
    RT = -np.sin(np.radians(2.0 * dtheta)) * RC
    tL, tC, tH = dL / SL, dC / SC, dH / SH
    return np.sqrt(np.maximum(0.0, tL * tL + tC * tC + tH * tH + RT * tC * tH))


def delta_e2000(img1, img2):
    """Per-pixel CIEDE2000 between two display-sRGB images [..., 3]."""
    return delta_e2000_lab(srgb_to_lab(img1), srgb_to_lab(img2))
