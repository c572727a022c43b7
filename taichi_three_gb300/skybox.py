"""Environment maps and image-based lighting (tina/skybox.py, tina/core/lighting.py).

Skybox keeps Tina's equirectangular layout: a (2*res, res) grid of RGB texels
indexed [i, j], looked up by spheremap + bilerp (tina/skybox.py:23-28, 138-145);
on the device it is a float16 (or float32) tensor of shape (2*res, res, 3).

SkyboxLighting shades with the environment instead of lamps.  mode='mc' is
the method's own Monte Carlo IBL: `spp` samples per pixel drawn by the
materials' importance samplers (tina/matr/material.py sample()), weight times
environment radiance (the estimator of tina/path/engine.py:243-266);
mode='mlp' uses a trained MLP-IBL network (taichi_three_gb300.mlp).  Empty
pixels show the environment along the view ray (Engine.render_background,
tina/core/engine.py:42-49).
"""
import numpy as np
import torch

from . import _native as N
from ._device import default_device, ptr


def unspheremap(coor):
    """Texel coordinate (v, u) in [0, 1]^2 -> direction (tina/skybox.py:31-36)."""
    v, u = coor[..., 0], coor[..., 1]
    h = u * 2 - 1
    r = np.sqrt(np.maximum(0.0, 1 - h * h))
    x, y = r * np.cos(v * 2 * np.pi), r * np.sin(v * 2 * np.pi)
    return np.stack([x, h, -y], axis=-1)  # dir.y, dir.z = dir.z, -dir.y


def texel_dirs(w, h):
    i, j = np.meshgrid(np.arange(w), np.arange(h), indexing='ij')
    coor = np.stack([i / (w - 1), j / (h - 1)], axis=-1)
    return unspheremap(coor)


def procedural_sky(res=512, nlobes=12, seed=0):
    """Seeded HDR environment, shape (2*res, res, 3) float32: a sky gradient over a
    darker ground plus `nlobes` Gaussian lobes (direction uniform on the sphere,
    angular width U[0.02, 0.3] rad, intensity lognormal(0, 1), slight tint)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = texel_dirs(2 * res, res)
    up = d[..., 1:2]
    horizon = np.array([0.60, 0.65, 0.70])
    zenith = np.array([0.20, 0.35, 0.75])
    ground = np.array([0.18, 0.16, 0.14])
    t = np.clip(up, 0.0, 1.0)
    sky = horizon * (1 - t) + zenith * t
    g = np.clip(-up * 8.0, 0.0, 1.0)
    img = sky * (1 - g) + ground * g
    dirs = rng.normal(size=(nlobes, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    widths = rng.uniform(0.02, 0.3, size=nlobes)
    inten = np.exp(rng.normal(0.0, 1.0, size=nlobes))
    tints = rng.uniform(0.6, 1.0, size=(nlobes, 3))
    for k in range(nlobes):
        cosang = np.clip(d @ dirs[k], -1.0, 1.0)
        ang = np.arccos(cosang)
        img = img + (inten[k] * np.exp(-0.5 * (ang / widths[k]) ** 2))[..., None] * tints[k]
    return img.astype(np.float32)


class Skybox:
    """An equirect environment map (tina/skybox.py:40-145).  `path` may be an int
    resolution (zeros), or an array of shape (2*res, res, 3)."""

    def __init__(self, path, scale=None, cubic=False, half=True):
        if cubic:
            raise NotImplementedError('cube-map skyboxes are not part of this build')
        if isinstance(path, int):
            img = np.zeros((2 * path, path, 3), np.float32)
        elif isinstance(path, (np.ndarray, torch.Tensor)):
            img = np.asarray(path.cpu() if isinstance(path, torch.Tensor) else path, np.float32)
        else:
            raise NotImplementedError('image decoding is not available; pass an array')
        if img.ndim != 3 or img.shape[2] != 3:
            raise ValueError('skybox arrays have shape (2*res, res, 3)')
        if scale is not None:
            img = img * scale
        self.shape = img.shape[:2]
        self.resolution = self.shape[1]
        self.half = half
        self.host = img
        self.img = torch.as_tensor(img, dtype=torch.float16 if half else torch.float32,
                                   device=default_device()).contiguous()

    def _t3_fill(self, lt, device, keep):
        lt.env = ptr(self.img, device, keep)
        lt.env_w, lt.env_h = self.shape
        lt.env_half = 1 if self.half else 0


class PlainSkybox(Skybox):
    """A uniform environment (tina/skybox.py:305-313)."""

    def __init__(self, color=(1.0, 1.0, 1.0)):
        c = np.broadcast_to(np.asarray(color, np.float32), (3,))
        super().__init__(np.tile(c, (8, 4, 1)), half=False)
        self.color = c


class SkyboxLighting:
    """IBL lighting: emission + environment integral (tina/core/lighting.py:5-21).

    mode 'mc': Monte Carlo with `spp` samples per pixel and stream `seed`;
    mode 'mlp': the trained network `mlp` (taichi_three_gb300.mlp.IBLNet).
    Extension: lamps added with add_light are summed on top (the reference's
    SkyboxLighting has none)."""

    def __init__(self, skybox=None, mode='mc', spp=256, seed=0, mlp=None):
        from .lighting import Lighting
        if skybox is None:
            skybox = Skybox(procedural_sky(64))
        if mode not in ('mc', 'mlp'):
            raise ValueError("mode must be 'mc' or 'mlp'")
        if mode == 'mlp' and mlp is None:
            raise ValueError("mode='mlp' needs a trained network (mlp=...)")
        self.skybox = skybox
        self.mode = mode
        self.spp = int(spp)
        self.seed = int(seed)
        self.mlp = mlp
        self._lamps = Lighting()

    # lamps (extension)
    def add_light(self, *args, **kwargs):
        return self._lamps.add_light(*args, **kwargs)

    def clear_lights(self):
        self._lamps.clear_lights()

    def set_ambient_light(self, color):
        pass  # SkyboxLighting has no ambient term

    def _t3_fill(self, lt):
        self._lamps._t3_fill(lt)
        for k in range(4):
            lt.ambient[k] = 0.0
        lt.mode = N.T3_LIGHT_IBL_MC if self.mode == 'mc' else N.T3_LIGHT_IBL_MLP
        lt.spp = self.spp
        lt.seed = self.seed & 0xFFFFFFFF

    def _t3_fill_device(self, lt, device, keep):
        self.skybox._t3_fill(lt, device, keep)
        if self.mode == 'mlp':
            lt.mlp = self.mlp.packed_ptr(device, keep)
