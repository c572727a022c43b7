"""MLP-IBL network kernels against the float64 numpy restatement.

CPU: the restatement's backward against central finite differences (pins the
checker itself).  GPU: feature encoding, forward, backward and Adam of the
CUDA kernels against it; tensor-core (BF16 tcgen05) inference against a numpy
emulation of BF16 operands with FP32 accumulation (checks the operand layout
and descriptors exactly) and against the FP32 path; a short training run
lowers the loss; checkpoint / resume round-trips.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def _params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    parts = []
    for fi, fo in ((MO.IN, MO.HID), (MO.HID, MO.HID), (MO.HID, MO.HID), (MO.HID, MO.OUT)):
        parts.append(rng.normal(0, np.sqrt(2.0 / fi) * scale, fi * fo))
        parts.append(rng.normal(0, 0.1, fo))
    return np.concatenate(parts)


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 2, 3))
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    return (d.reshape(n, 6).astype(np.float32), rng.uniform(0.05, 1, n).astype(np.float32),
            rng.uniform(0, 1, n).astype(np.float32))


def test_oracle_backward_matches_finite_differences():
    p = _params(0)
    nv, r, m = _inputs(7, 1)
    X = MO.encode(nv, r, m)
    T = np.random.default_rng(2).normal(size=(7, 9))
    g, _ = MO.backward(p, X, T)
    rng = np.random.default_rng(3)
    idx = np.concatenate([rng.choice(len(p), 40, replace=False), np.arange(len(p) - 16, len(p))])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        num = (MO.backward(p + e, X, T)[1] - MO.backward(p - e, X, T)[1]) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, num, g[i])


def test_oracle_encode_layout():
    X = MO.encode(np.array([[0.25, 0, 0, 0, 0, 0]]), np.array([0.5]), np.array([0.75]))
    # coordinate 0, frequency index f = o*4 + j at phase pi * 0.25 * 2^(o + j/4)
    assert np.isclose(X[0, 0], np.sin(np.pi * 0.25))
    assert np.isclose(X[0, 32 + 4], np.cos(np.pi * 0.25 * 2))
    assert X[0, 384] == 0.5 and X[0, 385] == 0.75 and not X[0, 386:].any()
    assert np.allclose(X[0, 64:96], 0) and np.allclose(X[0, 96:128], 1)


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def _bf16(x):
    """Round float32 to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _emulate_tc(p, X):
    """BF16 operands, high-precision accumulation, FP32 bias/ReLU, BF16 hidden."""
    W1, b1, W2, b2, W3, b3, W4, b4 = MO.unpack(p)
    h = _bf16(np.maximum((_bf16(X) @ _bf16(W1)).astype(np.float32) + b1.astype(np.float32), 0))
    h = _bf16(np.maximum((h @ _bf16(W2)).astype(np.float32) + b2.astype(np.float32), 0))
    h = _bf16(np.maximum((h @ _bf16(W3)).astype(np.float32) + b3.astype(np.float32), 0))
    return (h @ _bf16(W4)).astype(np.float32) + b4.astype(np.float32)


@pytest.fixture(scope='module')
def net(cuda):
    from taichi_three_gb300.mlp import IBLNet
    return IBLNet(seed=5)


@pytest.mark.gpu
def test_encode_matches_oracle(cuda, net):
    import torch
    nv, r, m = _inputs(1000, 11)
    X = net.encode(torch.from_numpy(nv).cuda(), torch.from_numpy(r).cuda(), torch.from_numpy(m).cuda())
    ref = MO.encode(nv.astype(np.float64), r, m)
    err = np.abs(X.cpu().numpy() - ref).max()
    # 8 double-angle steps amplify the base phase's rounding by up to 2^7
    assert err < 5e-4, err


@pytest.mark.gpu
def test_forward_backward_match_oracle(cuda, net):
    import torch
    B = 300  # not a multiple of the 64-row GEMM tile
    p = _params(7).astype(np.float32)
    nv, r, m = _inputs(B, 12)
    X = MO.encode(nv, r, m).astype(np.float32)
    T = np.random.default_rng(13).normal(size=(B, 9)).astype(np.float32)
    net.params = torch.from_numpy(p).cuda()
    Xd, Td = torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda()
    acts, Y = net.forward(Xd)
    _, Yref = MO.forward(p.astype(np.float64), X.astype(np.float64))
    assert np.abs(Y.cpu().numpy() - Yref).max() < 1e-4 * max(1.0, np.abs(Yref).max())
    g, loss = net.gradients(Xd, Td)
    gref, lref = MO.backward(p.astype(np.float64), X.astype(np.float64), T.astype(np.float64))
    g = g.cpu().numpy()
    assert abs(float(loss.item()) - lref) <= 1e-5 * lref
    scale = np.abs(gref).max()
    assert np.abs(g - gref).max() <= 1e-4 * scale, np.abs(g - gref).max() / scale


@pytest.mark.gpu
def test_adam_step_matches_numpy(cuda, net):
    import torch
    rng = np.random.default_rng(21)
    n = net.nparams
    p0 = rng.normal(size=n).astype(np.float32)
    g = rng.normal(size=n).astype(np.float32)
    net.params = torch.from_numpy(p0).cuda()
    net.m = torch.from_numpy(rng.normal(size=n).astype(np.float32) * 0.1).cuda()
    net.v = torch.from_numpy(rng.uniform(0, 0.1, n).astype(np.float32)).cuda()
    m0, v0 = net.m.cpu().numpy().astype(np.float64), net.v.cpu().numpy().astype(np.float64)
    net.step = 4
    net.adam_step(torch.from_numpy(g).cuda(), lr=1e-2)
    b1, b2, eps, t = 0.9, 0.999, 1e-8, 5
    m1 = b1 * m0 + (1 - b1) * g
    v1 = b2 * v0 + (1 - b2) * g.astype(np.float64) ** 2
    p1 = p0 - 1e-2 * (m1 / (1 - b1 ** t)) / (np.sqrt(v1 / (1 - b2 ** t)) + eps)
    assert np.abs(net.params.cpu().numpy() - p1).max() < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize('B', [1, 128, 1000, 152 * 128 * 2 + 37])
def test_tensor_core_inference(cuda, net, B):
    """B = 1 (one partial tile), 128, 1000 and > 2 tiles per CTA of the
    persistent 152-CTA grid."""
    import torch
    p = _params(9).astype(np.float32)
    net.params = torch.from_numpy(p).cuda()
    net._packed = None
    nv, r, m = _inputs(B, 14)
    Xd = net.encode(torch.from_numpy(nv).cuda(), torch.from_numpy(r).cuda(), torch.from_numpy(m).cuda())
    Ytc = net.infer(Xd, tensor_cores=True).cpu().numpy()
    Yf = net.infer(Xd, tensor_cores=False).cpu().numpy()
    X = Xd.cpu().numpy()
    emu = _emulate_tc(p.astype(np.float64), X)
    scale = max(1.0, np.abs(emu).max())
    d = np.abs(Ytc - emu)
    # rare one-ulp BF16 flips of a hidden unit are the only expected difference
    assert d.max() < 2e-2 * scale and d.mean() < 2e-4 * scale, (d.max(), d.mean())
    assert np.abs(Ytc - Yf).max() < 5e-2 * scale


@pytest.mark.gpu
def test_training_lowers_loss_and_checkpoint_roundtrip(cuda, tmp_path):
    import torch
    import taichi_three_gb300 as tina
    from taichi_three_gb300.mlp import IBLNet, sample_directions
    sky = tina.Skybox(tina.procedural_sky(32, seed=3))
    irr = IBLNet.irradiance_map(sky, res=(64, 32), spp=256)
    nv, r, m = sample_directions(8192, seed=4)
    T = IBLNet.targets(sky, irr, nv, r, spp=128)
    assert torch.isfinite(T).all() and (T >= 0).all()
    net = IBLNet(seed=1)
    X = net.encode(nv, r, m)
    _, l0 = net.gradients(X, T)
    net.fit(nv, r, m, T, steps=300, batch=2048, lr=2e-3)
    _, l1 = net.gradients(X, T)
    assert float(l1.item()) < 0.3 * float(l0.item()), (float(l0.item()), float(l1.item()))
    path = tmp_path / 'net.pt'
    net.save(path)
    net2 = IBLNet.load(path)
    assert net2.step == net.step and torch.equal(net2.params, net.params) and torch.equal(net2.v, net.v)
    assert torch.equal(net2.infer(X[:256]), net.infer(X[:256]))


@pytest.mark.gpu
def test_irradiance_of_uniform_sky_is_uniform(cuda):
    import taichi_three_gb300 as tina
    from taichi_three_gb300.mlp import IBLNet
    sky = tina.PlainSkybox((0.25, 0.5, 2.0))
    irr = IBLNet.irradiance_map(sky, res=(32, 16), spp=64).cpu().numpy()
    assert np.allclose(irr, [0.25, 0.5, 2.0], rtol=1e-5)
