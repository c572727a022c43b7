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
import ctypes as C

import numpy as np
import torch

from . import _native as N
from ._device import default_device, ptr, require_cuda


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


# CookTorrance.rough_levels (tina/matr/material.py:251-253)
ROUGH_LEVELS = [0.03, 0.08, 0.18, 0.35, 0.65, 1.0]


def rough_levels():
    """(level, step from the previous level) pairs, computed in Python floats
    as the reference does."""
    return [(a, a - b) for a, b in zip(ROUGH_LEVELS, [0] + ROUGH_LEVELS)]


def _cook_weights(nov, rough, n=1 << 16, seed=7):
    """E[Fc G] and E[G] of the reference's CookTorrance sampler
    (tina/matr/material.py:365-384, weight F * G) at NoV = nov, roughness
    `rough`, with Fc = (1 - VoH)^5; float64 Monte Carlo over fixed uniforms."""
    rng = np.random.Generator(np.random.PCG64(seed))
    u, v = rng.random(n), rng.random(n)
    a2 = max(0.0, rough ** 2)
    h = np.sqrt((1 - u) / (1 - u * (1 - a2)))
    V = np.array([np.sqrt(max(0.0, 1 - nov * nov)), 0.0, nov])
    nrm = np.array([0.0, 0.0, 1.0])
    rdir = -V - 2 * np.dot(nrm, -V) * nrm
    bitan = np.cross(rdir, [233.0, 666.0, 512.0])
    bitan /= np.linalg.norm(bitan)
    tan = np.cross(bitan, rdir)
    r = np.sqrt(np.maximum(0.0, 1 - h * h))
    odir = (r * np.cos(2 * np.pi * v))[:, None] * tan + (r * np.sin(2 * np.pi * v))[:, None] * bitan + \
        h[:, None] * rdir
    half = V + odir
    half /= np.linalg.norm(half, axis=1, keepdims=True)
    eps = 1e-10
    NoL = max(eps, float(np.dot(V, nrm)))
    NoV = np.maximum(eps, odir @ nrm)
    VoH = np.minimum(1 - eps, np.maximum(eps, np.sum(half * odir, axis=1)))
    alpha2 = max(1e-6, rough ** 2)
    k = alpha2 / 2
    G = 1 / ((NoV * k + 1 - k) * (NoL * k + 1 - k)) / ((1 - alpha2) + 4 * np.pi * alpha2)
    G = np.where(odir @ nrm < 0, 0.0, G)  # the sampler zeroes F below the surface
    Fc = (1 - VoH) ** 5
    return float(np.mean(Fc * G)), float(np.mean(G))


def split_sum_lut():
    """This build's own split-sum table for CookTorrance.sample_ibl: texel
    (i, j) holds (A, B) with f0 * A + B = E[F G] of the reference's own
    sampler at NoV = i and roughness = j (clamped to [1e-3, 1] and [0, 1]),
    float32 [3, 3, 2].  The reference reads its table (the image
    assets/lut.jpg, which cannot be decoded here) at (VoH, roughness) in texel
    units, i.e. only the texels this table holds."""
    lut = np.zeros((3, 3, 2), np.float64)
    for i in range(3):
        for j in range(3):
            b, g = _cook_weights(min(max(float(i), 1e-3), 1.0), min(float(j), 1.0))
            lut[i, j] = (g - b, b)
    return lut.astype(np.float32)


class IBLTables:
    """SkyboxLighting's prefiltered tables (tina/matr/material.py:279-316,
    :407-438), baked on the device by t3_ibl_bake: the environment, then one
    map per roughness level (resolution divided by 2^(4 step), samples per
    texel 8 * precision growing by 3^(4 step) per level, as the reference
    sizes them; at least 2 x 2 texels), the Lambert map at resolution / 6 with
    128 * precision samples (the reference also runs a KNN denoiser over it,
    which is not restated), and the split-sum LUT."""

    def __init__(self, skybox, precision=32, seed=0, lut=None):
        require_cuda('IBLTables')
        lib = N.load()
        dev = default_device()
        keep = []
        env = ptr(skybox.img, dev, keep)
        stream = torch.cuda.current_stream().cuda_stream

        def bake(rough, nsamples, res, k):
            out = torch.empty((2 * res, res, 3), dtype=torch.float32, device=dev)
            N.check(lib.t3_ibl_bake(env, skybox.shape[0], skybox.shape[1], int(skybox.half), float(rough),
                                    int(nsamples), (seed * 7919 + k) & 0xFFFFFFFF, out.data_ptr(),
                                    out.shape[0], out.shape[1], stream), 't3_ibl_bake')
            return out

        self.spec = [skybox.img]
        self.spec_half = [bool(skybox.half)]
        resolution = skybox.resolution
        nsamples = 8 * precision
        for k, (rough, step) in enumerate(rough_levels()):
            resolution = int(resolution / 2 ** (step * 4))
            self.spec.append(bake(rough, nsamples, max(resolution, 2), k + 1))
            self.spec_half.append(False)
            nsamples = int(nsamples * 3 ** (step * 4))
        self.diffuse = bake(-1.0, 128 * precision, max(skybox.resolution // 6, 2), 0)
        table = split_sum_lut() if lut is None else np.asarray(lut, np.float32)
        if table.ndim != 3 or table.shape[2] < 2 or table.shape[0] < 2 or table.shape[1] < 2:
            raise ValueError('the LUT is an array [w >= 2, h >= 2, >= 2 channels]')
        self.lut = torch.as_tensor(np.ascontiguousarray(table[..., :2]), device=dev)
        del keep

    def _t3_tables(self, device, keep):
        T = N.t3_ibl_tables()
        for k, (img, half) in enumerate(zip(self.spec, self.spec_half)):
            T.spec[k].data = ptr(img, device, keep)
            T.spec[k].w, T.spec[k].h = img.shape[0], img.shape[1]
            T.spec[k].half = int(half)
        T.diffuse.data = ptr(self.diffuse, device, keep)
        T.diffuse.w, T.diffuse.h = self.diffuse.shape[0], self.diffuse.shape[1]
        T.lut = ptr(self.lut, device, keep)
        T.lut_w, T.lut_h = self.lut.shape[0], self.lut.shape[1]
        keep.append(T)
        return T


class SkyboxLighting:
    """IBL lighting: emission + environment integral (tina/core/lighting.py:5-21).

    mode 'prefiltered' (the reference's SkyboxLighting): the materials'
    sample_ibl lookups of tables baked from the skybox (IBLTables, baked on
    first use with `precision` as in the reference);
    mode 'mc': the method's own Monte Carlo IBL with `spp` samples per pixel
    and stream `seed`;
    mode 'mlp': the trained network `mlp` (taichi_three_gb300.mlp.IBLNet).
    Extension: lamps added with add_light are summed on top (the reference's
    SkyboxLighting has none)."""

    def __init__(self, skybox=None, mode='prefiltered', spp=256, seed=0, mlp=None, precision=32,
                 ibltab=None):
        from .lighting import Lighting
        if skybox is None:
            skybox = Skybox(procedural_sky(64))
        if mode not in ('prefiltered', 'mc', 'mlp'):
            raise ValueError("mode must be 'prefiltered', 'mc' or 'mlp'")
        if mode == 'mlp' and mlp is None:
            raise ValueError("mode='mlp' needs a trained network (mlp=...)")
        self.skybox = skybox
        self.mode = mode
        self.spp = int(spp)
        self.seed = int(seed)
        self.mlp = mlp
        self.precision = int(precision)
        self.ibltab = ibltab  # IBLTables, baked on first use when None
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
        lt.mode = {'mc': N.T3_LIGHT_IBL_MC, 'mlp': N.T3_LIGHT_IBL_MLP,
                   'prefiltered': N.T3_LIGHT_IBL_PREFILTERED}[self.mode]
        lt.spp = self.spp
        lt.seed = self.seed & 0xFFFFFFFF

    def _t3_fill_device(self, lt, device, keep):
        self.skybox._t3_fill(lt, device, keep)
        if self.mode == 'mlp':
            lt.mlp = self.mlp.packed_ptr(device, keep)
        if self.mode == 'prefiltered':
            if self.ibltab is None:
                self.ibltab = IBLTables(self.skybox, self.precision, self.seed)
            T = self.ibltab._t3_tables(device, keep)
            lt.tables = C.pointer(T)
