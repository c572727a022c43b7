"""Material parameter nodes (tina/matr/nodes.py).

A node is compiled into one entry of the material expression table that the
CUDA shade kernel evaluates once per pixel.  Argument coercion follows
Node.__init__ (tina/matr/nodes.py:9-33): int/float -> Const, list/tuple ->
vector Const, str -> Input (an image path -> Texture).
"""
import numbers

import numpy as np


class Node:
    arguments = []
    defaults = []

    def __init__(self, **kwargs):
        # Contract of the reference's keyword binding: every declared argument
        # takes the caller's value or its default; a None default means the
        # argument is required (ValueError when absent); any keyword the node
        # does not declare is a TypeError.  Required arguments are checked
        # before unknown keywords, as there.
        table = dict(zip(self.arguments, self.defaults))
        missing = [k for k, d in table.items() if d is None and k not in kwargs]
        if missing:
            raise ValueError(f'`{missing[0]}` must specified for `{type(self)}`')
        unknown = [k for k in kwargs if k not in table]
        if unknown:
            raise TypeError(
                f"{type(self).__name__}() got an unexpected keyword argument '{unknown[0]}', "
                f"supported keywords are: {self.arguments}")
        self.params = {k: as_node(kwargs.get(k, d)) for k, d in table.items()}

    def param(self, key):
        return self.params[key]


def as_node(value):
    if isinstance(value, Node):
        return value
    if isinstance(value, (bool, np.bool_)):
        return Const(float(value))
    if isinstance(value, numbers.Number):
        return Const(value)
    if isinstance(value, (list, tuple, np.ndarray)):
        return Const(tuple(float(v) for v in np.asarray(value).ravel()))
    if isinstance(value, str):
        if any(value.endswith(x) for x in ['.png', '.jpg', '.bmp']):
            return Texture(value)
        return Input(value)
    raise TypeError(f'cannot use {value!r} as a material parameter')


class Const(Node):
    """A constant scalar or 3-vector (tina/matr/nodes.py:42-49).  A Python int
    keeps its integer-ness: Tina raises to an int power by repeated squaring."""

    def __init__(self, value):  # noqa: super not called, like the reference
        self.params = {}
        if isinstance(value, (tuple, list, np.ndarray)):
            v = tuple(float(x) for x in np.asarray(value).ravel())
            if len(v) == 1:
                v = v[0]
            elif len(v) != 3:
                raise ValueError(f'Const vectors must have 1 or 3 entries, got {len(v)}')
        else:
            v = value
        self.value = v

    @property
    def is_int(self):
        return isinstance(self.value, numbers.Integral) and not isinstance(self.value, bool)


class Param(Node):
    """A run-time adjustable value (tina/matr/nodes.py:52-68); set `.value` (or
    call set()) between frames.  GUI sliders are not part of this build."""

    def __init__(self, dtype=float, dim=None, initial=0):
        self.params = {}
        self.dtype = dtype
        self.dim = dim
        self.initial = initial
        self.value = initial

    def set(self, value):
        self.value = value


class Input(Node):
    """Per-fragment inputs 'pos', 'color', 'normal', 'texcoord'
    (tina/matr/nodes.py:79-96); 'color' is always (1, 1, 1) on the triangle path
    (tina/core/triangle.py:48)."""
    NAMES = {'pos': 0, 'color': 1, 'normal': 2, 'texcoord': 3}

    def __init__(self, name):
        self.params = {}
        if name not in self.NAMES:
            raise ValueError(f'unknown Input {name!r}; expected one of {list(self.NAMES)}')
        self.name = name


class FaceAttr(Node):
    """Extension node: a per-face material parameter read from the mesh's
    face attribute table (`mesh.set_face_attrs(array[nfaces, C])`), channels
    [channel, channel + width).  The reference has no per-face parameters on the
    raster path; with constant attributes it reduces to Const."""

    def __init__(self, channel, width=1):
        self.params = {}
        if width not in (1, 3):
            raise ValueError('FaceAttr width must be 1 or 3')
        self.channel = int(channel)
        self.width = int(width)


class Texture(Node):
    """Image texture (tina/matr/nodes.py:99-111, advans.py:8-28): an array
    [w, h] or [w, h, 3] indexed [i, j] like a Taichi field (uint8 is scaled by
    1/255), or a .npy path; sampled with bilerp at texcoord * (shape - 1).
    Image-file decoding is not part of this build (pass the decoded array)."""
    arguments = ['texcoord']
    defaults = ['texcoord']

    def __init__(self, path, **kwargs):
        import torch
        from ._device import default_device
        if isinstance(path, str):
            if not path.endswith('.npy'):
                raise NotImplementedError('image decoding is not available here; pass the image as an '
                                          'array (or a .npy file)')
            img = np.load(path)
        else:
            img = np.asarray(path.cpu() if hasattr(path, 'cpu') else path)
        if img.dtype == np.uint8:
            img = img / 255
        img = np.asarray(img, np.float32)
        if img.ndim == 3 and img.shape[2] == 1:
            img = img[..., 0]
        if img.ndim not in (2, 3) or (img.ndim == 3 and img.shape[2] != 3):
            raise ValueError('textures are [w, h] or [w, h, 3] arrays')
        super().__init__(**kwargs)
        self.shape = img.shape[:2]
        self.channels = 1 if img.ndim == 2 else 3
        self.data = torch.as_tensor(np.ascontiguousarray(img), device=default_device())


class ChessboardTexture(Node):
    """lerp((texcoord // size).sum() % 2, color0, color1) (tina/matr/nodes.py:114-126)."""
    arguments = ['texcoord', 'size', 'color0', 'color1']
    defaults = ['texcoord', 0.1, 0.4, 0.9]
