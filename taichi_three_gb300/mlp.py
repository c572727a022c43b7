"""MLP-IBL: a small network that stands in for the IBL integral.

The network (400 -> 64 -> 64 -> 64 -> 16, ReLU) maps Fourier features of the
shading normal and view direction plus roughness and metallic to log1p of
the albedo-independent IBL integrals of the Lambert and CookTorrance lobes
(E_d, S1, S2; RGB each) under the method's own Monte Carlo estimator;
shading composes them with each pixel's albedo, f0 and lobe weights.  It is
trained on the GPU by the library's own kernels (t3_mlp_targets / encode /
forward / backward / adam) on targets integrated by Monte Carlo from the
environment map, and runs at render time on the tensor cores (BF16 operands,
FP32 accumulation) fused into the shading kernel.
"""
import math

import torch

from . import _native as N
from ._device import default_device, ptr, require_cuda


def _stream():
    return torch.cuda.current_stream().cuda_stream


def sample_directions(n, seed=0, device=None):
    """Training inputs: normals and view directions uniform on the sphere (the
    soup's shading normals are random unit vectors), roughness U[0.05, 1],
    metallic U[0, 1].  Returns nv [n, 6], rough [n], metal [n]."""
    device = device or default_device()
    g = torch.Generator(device='cpu').manual_seed(seed)
    d = torch.randn(n, 2, 3, generator=g)
    d = d / d.norm(dim=-1, keepdim=True)
    rough = torch.rand(n, generator=g) * 0.95 + 0.05
    metal = torch.rand(n, generator=g)
    return (d.reshape(n, 6).to(device).contiguous(), rough.to(device).contiguous(),
            metal.to(device).contiguous())


class IBLNet:
    IN, HID, OUT = N.T3_MLP_IN, N.T3_MLP_HID, N.T3_MLP_OUT

    def __init__(self, seed=0, device=None):
        self.device = device or default_device()
        lib = N.load()
        self.nparams = int(lib.t3_mlp_param_count())
        g = torch.Generator(device='cpu').manual_seed(seed)
        parts = []
        for fan_in, fan_out in ((self.IN, self.HID), (self.HID, self.HID), (self.HID, self.HID),
                                (self.HID, self.OUT)):
            parts.append(torch.randn(fan_in * fan_out, generator=g) * math.sqrt(2.0 / fan_in))
            parts.append(torch.zeros(fan_out))
        self.params = torch.cat(parts).to(self.device).contiguous()
        assert self.params.numel() == self.nparams
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self._packed = None

    # -- data ------------------------------------------------------------------
    @staticmethod
    def irradiance_map(skybox, res=(256, 128), spp=4096, seed=1):
        require_cuda('IBLNet.irradiance_map')
        lib = N.load()
        keep = []
        env = ptr(skybox.img, 'cuda', keep)
        m = torch.empty((res[0], res[1], 3), dtype=torch.float32, device='cuda')
        N.check(lib.t3_mlp_irradiance_map(env, skybox.shape[0], skybox.shape[1], int(skybox.half),
                                          res[0], res[1], spp, seed, m.data_ptr(), _stream()),
                't3_mlp_irradiance_map')
        return m

    @staticmethod
    def targets(skybox, irr, nv, rough, spp=4096, seed=2, chunk=1 << 20):
        """log1p(E_d, S1, S2) [n, 9] by Monte Carlo (spp samples per target)."""
        lib = N.load()
        keep = []
        env = ptr(skybox.img, 'cuda', keep)
        n = nv.shape[0]
        t = torch.empty((n, 9), dtype=torch.float32, device='cuda')
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            N.check(lib.t3_mlp_targets(env, skybox.shape[0], skybox.shape[1], int(skybox.half),
                                       irr.data_ptr(), irr.shape[0], irr.shape[1],
                                       nv[s:].data_ptr(), rough[s:].data_ptr(), e - s, spp,
                                       seed + s, t[s:].data_ptr(), _stream()), 't3_mlp_targets')
        return t

    def encode(self, nv, rough, metal):
        lib = N.load()
        n = nv.shape[0]
        X = torch.empty((n, self.IN), dtype=torch.float32, device=nv.device)
        N.check(lib.t3_mlp_encode(nv.data_ptr(), rough.data_ptr(),
                                  metal.data_ptr() if metal is not None else None, n, X.data_ptr(),
                                  _stream()), 't3_mlp_encode')
        return X

    # -- training ---------------------------------------------------------------
    def forward(self, X):
        lib = N.load()
        B = X.shape[0]
        acts = torch.empty((B, 3 * self.HID), dtype=torch.float32, device=X.device)
        Y = torch.empty((B, self.OUT), dtype=torch.float32, device=X.device)
        N.check(lib.t3_mlp_forward(self.params.data_ptr(), X.data_ptr(), B, acts.data_ptr(),
                                   Y.data_ptr(), _stream()), 't3_mlp_forward')
        return acts, Y

    def gradients(self, X, T):
        """(gradient in the parameter layout, mean squared error) of a batch."""
        lib = N.load()
        B = X.shape[0]
        acts, Y = self.forward(X)
        grads = torch.empty_like(self.params)
        dbuf = torch.empty((B, 2 * self.HID + self.OUT), dtype=torch.float32, device=X.device)
        loss = torch.zeros(1, dtype=torch.float32, device=X.device)
        N.check(lib.t3_mlp_backward(self.params.data_ptr(), X.data_ptr(), acts.data_ptr(),
                                    Y.data_ptr(), T.data_ptr(), B, grads.data_ptr(),
                                    dbuf.data_ptr(), loss.data_ptr(), _stream()), 't3_mlp_backward')
        return grads, loss

    def adam_step(self, grads, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        lib = N.load()
        self.step += 1
        N.check(lib.t3_mlp_adam(self.params.data_ptr(), grads.data_ptr(), self.m.data_ptr(),
                                self.v.data_ptr(), self.nparams, lr, beta1, beta2, eps, self.step,
                                _stream()), 't3_mlp_adam')
        self._packed = None

    def fit(self, nv, rough, metal, targets, steps=1000, batch=16384, lr=2e-3, lr_end=1e-4,
            seed=0, log_every=0):
        """Adam on minibatches drawn from the training set; cosine-decayed lr.
        Returns the list of batch losses (device floats read every log_every)."""
        n = nv.shape[0]
        g = torch.Generator(device='cpu').manual_seed(seed)
        losses = []
        for it in range(steps):
            idx = torch.randint(0, n, (batch,), generator=g).to(nv.device)
            X = self.encode(nv[idx].contiguous(), rough[idx].contiguous(), metal[idx].contiguous())
            grads, loss = self.gradients(X, targets[idx].contiguous())
            a = lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * it / max(1, steps)))
            self.adam_step(grads, lr=a)
            if log_every and (it % log_every == 0 or it == steps - 1):
                losses.append((it, float(loss.item())))
        return losses

    # -- inference ----------------------------------------------------------------
    def pack(self):
        """The BF16 tensor-core blob (cached until the next update)."""
        if self._packed is None:
            lib = N.load()
            nb = int(lib.t3_mlp_packed_bytes())
            blob = torch.zeros(nb, dtype=torch.uint8, device=self.params.device)
            N.check(lib.t3_mlp_pack(self.params.data_ptr(), blob.data_ptr(), _stream()), 't3_mlp_pack')
            self._packed = blob
        return self._packed

    def packed_ptr(self, device, keep):
        return ptr(self.pack(), device, keep)

    def infer(self, X, tensor_cores=True):
        lib = N.load()
        B = X.shape[0]
        Y = torch.empty((B, self.OUT), dtype=torch.float32, device=X.device)
        if tensor_cores:
            status = torch.zeros(1, dtype=torch.int32, device=X.device)
            N.check(lib.t3_mlp_infer(self.pack().data_ptr(), X.data_ptr(), B, Y.data_ptr(),
                                     status.data_ptr(), _stream()), 't3_mlp_infer')
            if int(status.item()) != 0:
                raise RuntimeError(f'MLP inference reported device status {int(status.item())}')
        else:
            N.check(lib.t3_mlp_infer_f32(self.params.data_ptr(), X.data_ptr(), B, Y.data_ptr(),
                                         _stream()), 't3_mlp_infer_f32')
        return Y

    # -- checkpoint / resume --------------------------------------------------------
    def state_dict(self):
        return {'params': self.params.detach().cpu(), 'm': self.m.cpu(), 'v': self.v.cpu(),
                'step': self.step}

    def load_state_dict(self, d):
        self.params = d['params'].to(self.device).contiguous()
        self.m = d['m'].to(self.device).contiguous()
        self.v = d['v'].to(self.device).contiguous()
        self.step = int(d['step'])
        self._packed = None

    def save(self, path):
        torch.save(self.state_dict(), path)

    @classmethod
    def load(cls, path, device=None):
        net = cls(device=device)
        net.load_state_dict(torch.load(path, map_location='cpu'))
        return net


def train_for_skybox(skybox, samples=1 << 24, spp=4096, steps=4000, batch=16384, lr=2e-3,
                     lr_end=5e-5, irr_res=(256, 128), irr_spp=4096, seed=0, net=None, log_every=0):
    """Trains an IBLNet for `skybox`: an irradiance map (irr_spp cosine samples
    per texel), `samples` random (n, v, roughness, metallic) inputs with
    spp-sample Monte Carlo targets, then `steps` Adam steps.  Returns
    (net, losses)."""
    irr = IBLNet.irradiance_map(skybox, res=irr_res, spp=irr_spp, seed=seed + 1)
    nv, rough, metal = sample_directions(samples, seed=seed)
    T = IBLNet.targets(skybox, irr, nv, rough, spp=spp, seed=seed + 2)
    net = net or IBLNet(seed=seed)
    losses = net.fit(nv, rough, metal, T, steps=steps, batch=batch, lr=lr, lr_end=lr_end, seed=seed,
                     log_every=log_every)
    return net, losses
