"""Test infrastructure only: numpy float32 restatement of the post-processing
passes (tina/postp/blooming.py:52-75 with init_gwei :30-40,
tina/postp/fxaa.py:25-68, tina/util/accumator.py:16-23) on [W, H, 3] images,
with out-of-image reads clamped (the kernels' documented choice)."""
import numpy as np

f32 = np.float32


def _bilerp(img, px, py):
    w, h = img.shape[:2]
    fx, fy = np.floor(px), np.floor(py)
    ix, iy = fx.astype(np.int64), fy.astype(np.int64)
    x0, x1 = (px - fx).astype(f32), (py - fy).astype(f32)
    y0, y1 = f32(1) - x0, f32(1) - x1

    def at(i, j):
        return img[np.clip(i, 0, w - 1), np.clip(j, 0, h - 1)]
    r = at(ix + 1, iy + 1) * (x0 * x1)[..., None]
    r = r + at(ix + 1, iy) * (x0 * y1)[..., None]
    r = r + at(ix, iy) * (y0 * y1)[..., None]
    r = r + at(ix, iy + 1) * (y0 * x1)[..., None]
    return r.astype(f32)


def bloom(img, thresh=1.0, factor=1.0, scale=0.25, sigma=1.0, radius=None):
    img = np.asarray(img, f32).copy()
    W, H = img.shape[:2]
    radius = radius or min(W, H) // 16
    g = np.empty(radius + 1, f32)
    s = f32(-1)
    for i in range(radius + 1):
        x = f32(sigma) * f32(i) / f32(radius)
        g[i] = np.exp(-(x * x), dtype=f32)
        s = f32(s + g[i] * f32(2))
    g = (g / s).astype(f32)
    t = np.maximum(f32(0), img - f32(thresh))
    t = f32(1) - f32(1) / (f32(1) + f32(scale) * t)
    filt = (f32(factor) * t).astype(f32)
    w, h = W // 2, H // 2
    half = ((filt[0:2 * w:2, 0:2 * h:2] + filt[0:2 * w:2, 1:2 * h:2]) + filt[1:2 * w:2, 0:2 * h:2]
            + filt[1:2 * w:2, 1:2 * h:2]) / f32(4)
    half = half.astype(f32)
    xs, ys = np.arange(w), np.arange(h)
    tmp = half * g[0]
    for k in range(1, radius + 1):
        tmp = tmp + (half[np.maximum(0, xs - k)] + half[np.minimum(w - 1, xs + k)]) * g[k]
    out = tmp * g[0]
    for k in range(1, radius + 1):
        out = out + (tmp[:, np.maximum(0, ys - k)] + tmp[:, np.minimum(h - 1, ys + k)]) * g[k]
    X, Y = np.meshgrid(np.arange(W), np.arange(H), indexing='ij')
    return (img + _bilerp(out.astype(f32), X.astype(f32) / f32(2), Y.astype(f32) / f32(2))).astype(f32)


def fxaa(img, abs_thresh=0.0625, rel_thresh=0.063, factor=1.0):
    img = np.asarray(img, f32)
    W, H = img.shape[:2]
    lumi = np.clip((f32(0.2989) * img[..., 0] + f32(0.587) * img[..., 1]) + f32(0.114) * img[..., 2], 0, 1)
    X, Y = np.meshgrid(np.arange(W), np.arange(H), indexing='ij')

    def L(dx, dy):
        return lumi[np.clip(X + dx, 0, W - 1), np.clip(Y + dy, 0, H - 1)]
    m, n, e, s, w = L(0, 0), L(0, 1), L(1, 0), L(0, -1), L(-1, 0)
    ne, nw, se, sw = L(1, 1), L(-1, 1), L(1, -1), L(-1, -1)
    hi = np.maximum.reduce([m, n, e, s, w])
    lo = np.minimum.reduce([m, n, e, s, w])
    c = hi - lo
    skip = (c < f32(abs_thresh)) | (c < f32(rel_thresh) * hi)
    filt = f32(2) * (((n + e) + s) + w)
    filt = filt + (((ne + nw) + se) + sw)
    filt = np.abs(filt / f32(12) - m)
    with np.errstate(divide='ignore', invalid='ignore'):
        filt = np.clip(filt / c, 0, 1)
    sm = (filt * filt) * (f32(3) - f32(2) * filt)
    blend = (sm * sm) * f32(factor)
    def edge(a, b, mid):
        return np.abs((a + b) - f32(2) * mid)
    hori = (edge(n, s, m) * f32(2) + edge(ne, se, e)) + edge(nw, sw, w)
    vert = (edge(e, w, m) * f32(2) + edge(ne, nw, n)) + edge(se, sw, s)
    is_hori = hori >= vert
    pl = np.where(is_hori, n, e)
    nl = np.where(is_hori, s, w)
    blend = np.where(np.abs(pl - m) < np.abs(nl - m), -blend, blend)
    blend = np.where(skip, f32(0), blend)  # skipped pixels keep their colour (their blend is unused)
    px = X.astype(f32) + np.where(is_hori, f32(0), blend)
    py = Y.astype(f32) + np.where(is_hori, blend, f32(0))
    out = _bilerp(img, px, py)
    return np.where(skip[..., None], img, out).astype(f32)


def accumulate(acc, src, count):
    inv = f32(1) / f32(count)
    return (np.asarray(acc, f32) * (f32(1) - inv) + np.asarray(src, f32) * inv).astype(f32)
