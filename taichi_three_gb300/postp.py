"""Post-processing on scene.img: the ACES tonemap (tina/postp/tonemap.py).
Scene.render applies it inside the shade kernel's epilogue; ToneMapping.apply
is the standalone in-place pass on a device image."""
import torch

from . import _native as N
from ._device import require_cuda


def aces_tonemap(color):
    """c * (2.51 c + 0.03) / (c * (2.43 c + 0.59) + 0.14) (tina/advans.py:32-34),
    on numbers or tensors (host-side helper for inspection)."""
    return color * (2.51 * color + 0.03) / (color * (2.43 * color + 0.59) + 0.14)


class ToneMapping:
    def __init__(self, res):
        self.res = res

    def apply(self, image):
        require_cuda('ToneMapping.apply')
        lib = N.load()
        if image.dtype != torch.float32 or not image.is_contiguous():
            raise ValueError('ToneMapping.apply needs a contiguous float32 device image')
        N.check(lib.t3_tonemap(image.data_ptr(), image.numel(), torch.cuda.current_stream().cuda_stream),
                't3_tonemap')


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _check_image(image, name):
    if image.dtype != torch.float32 or not image.is_contiguous() or image.dim() != 3 or image.shape[2] != 3:
        raise ValueError(f'{name} needs a contiguous float32 (W, H, 3) device image')


class Blooming:
    """Blooming (tina/postp/blooming.py): thresh 1, factor 1, scale 0.25,
    sigma 1, radius min(res) // 16; apply(image) works in place on the HDR
    image (Scene.render runs it before the tonemap)."""

    def __init__(self, res):
        self.res = tuple(res) if not isinstance(res, int) else (res, res)
        self.thresh, self.factor, self.scale, self.sigma = 1.0, 1.0, 0.25, 1.0
        self.radius = min(*self.res) // 16
        self._ws = None

    def apply(self, image):
        require_cuda('Blooming.apply')
        _check_image(image, 'Blooming.apply')
        lib = N.load()
        W, H = image.shape[:2]
        n = lib.t3_bloom_workspace_floats(W, H)
        if self._ws is None or self._ws.numel() < n:
            self._ws = torch.empty(max(n, 1), dtype=torch.float32, device=image.device)
        N.check(lib.t3_bloom(image.data_ptr(), W, H, self.thresh, self.factor, self.scale, self.sigma,
                             max(1, min(128, self.radius)), self._ws.data_ptr(), self._ws.numel(),
                             _stream()), 't3_bloom')


class FXAA:
    """FXAA (tina/postp/fxaa.py): abs_thresh 0.0625, rel_thresh 0.063,
    factor 1; apply(image) in place."""

    def __init__(self, res):
        self.res = tuple(res) if not isinstance(res, int) else (res, res)
        self.abs_thresh, self.rel_thresh, self.factor = 0.0625, 0.063, 1.0
        self._ws = None

    def apply(self, image):
        require_cuda('FXAA.apply')
        _check_image(image, 'FXAA.apply')
        lib = N.load()
        W, H = image.shape[:2]
        n = lib.t3_fxaa_workspace_floats(W, H)
        if self._ws is None or self._ws.numel() < n:
            self._ws = torch.empty(n, dtype=torch.float32, device=image.device)
        N.check(lib.t3_fxaa(image.data_ptr(), W, H, self.abs_thresh, self.rel_thresh, self.factor,
                            self._ws.data_ptr(), self._ws.numel(), _stream()), 't3_fxaa')


class Accumator:
    """Temporal accumulation (tina/util/accumator.py): img = running mean of
    the frames passed to update(); clear() restarts it."""

    def __init__(self, res):
        self.res = tuple(res) if not isinstance(res, int) else (res, res)
        self.img = None
        self.count = 0

    def clear(self):
        self.count = 0
        if self.img is not None:
            self.img.zero_()

    def update(self, src):
        require_cuda('Accumator.update')
        _check_image(src, 'Accumator.update')
        if self.img is None or self.img.shape != src.shape:
            self.img = torch.zeros_like(src)
        self.count += 1
        N.check(N.load().t3_accumulate(self.img.data_ptr(), src.data_ptr(), src.numel(), self.count,
                                       _stream()), 't3_accumulate')
