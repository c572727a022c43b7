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
