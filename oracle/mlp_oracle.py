"""Test infrastructure only: a float64 numpy restatement of the MLP-IBL
network (feature encoding, forward, backward of the mean squared error, Adam)
used to check the CUDA kernels' gradients and outputs."""
import numpy as np

IN, HID, OUT = 400, 64, 16


def encode(nv, rough, metal):
    """Features [B, 400]: sin / cos of pi * c * 2^(o + j/4), o = 0..7, j = 0..3,
    per coordinate of n and of r = 2 (n . v) n - v, then roughness, metallic,
    zeros."""
    nv = np.asarray(nv, np.float64)
    n, v = nv[:, :3], nv[:, 3:]
    nv = np.concatenate([n, 2 * (n * v).sum(1, keepdims=True) * n - v], axis=1)
    B = nv.shape[0]
    X = np.zeros((B, IN))
    for c in range(6):
        for j in range(4):
            for o in range(8):
                f = o * 4 + j
                a = np.pi * nv[:, c] * 2.0 ** (o + j / 4)
                X[:, c * 64 + f] = np.sin(a)
                X[:, c * 64 + 32 + f] = np.cos(a)
    X[:, 384] = rough
    X[:, 385] = metal
    return X


def unpack(p):
    p = np.asarray(p, np.float64)
    sizes = [(IN, HID), (HID,), (HID, HID), (HID,), (HID, HID), (HID,), (HID, OUT), (OUT,)]
    out, o = [], 0
    for s in sizes:
        n = int(np.prod(s))
        out.append(p[o:o + n].reshape(s))
        o += n
    return out


def forward(p, X):
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p)
    h1 = np.maximum(X @ W1 + b1, 0)
    h2 = np.maximum(h1 @ W2 + b2, 0)
    h3 = np.maximum(h2 @ W3 + b3, 0)
    return (h1, h2, h3), h3 @ W4 + b4


def backward(p, X, T):
    """Gradient (parameter layout) and loss = mean over batch and 9 outputs of (y - t)^2."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(p)
    (h1, h2, h3), Y = forward(p, X)
    B = X.shape[0]
    d = np.zeros_like(Y)
    d[:, :9] = Y[:, :9] - T
    loss = (d[:, :9] ** 2).sum() / (B * 9)
    dY = 2 * d / (B * 9)
    gW4, gb4 = h3.T @ dY, dY.sum(0)
    dh3 = (dY @ W4.T) * (h3 > 0)
    gW3, gb3 = h2.T @ dh3, dh3.sum(0)
    dh2 = (dh3 @ W3.T) * (h2 > 0)
    gW2, gb2 = h1.T @ dh2, dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (h1 > 0)
    gW1, gb1 = X.T @ dh1, dh1.sum(0)
    g = np.concatenate([a.ravel() for a in (gW1, gb1, gW2, gb2, gW3, gb3, gW4, gb4)])
    return g, loss
