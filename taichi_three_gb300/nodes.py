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
        self.params = {}
        for dfl, key in zip(self.defaults, self.arguments):
            if key not in kwargs:
                if dfl is None:
                    raise ValueError(f'`{key}` must specified for `{type(self)}`')
                value = dfl
            else:
                value = kwargs[key]
                del kwargs[key]
            self.params[key] = as_node(value)
        for key in kwargs.keys():
            raise TypeError(
                f"{type(self).__name__}() got an unexpected keyword argument '{key}', "
                f"supported keywords are: {self.arguments}")

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
    """Image texture node (tina/matr/nodes.py:99-111): not part of this build."""

    def __init__(self, path, **kwargs):
        raise NotImplementedError('Texture nodes are not implemented by this rasteriser build')


class ChessboardTexture(Node):
    def __init__(self, **kwargs):
        raise NotImplementedError('ChessboardTexture is not implemented by this rasteriser build')
