"""Materials (tina/matr/material.py) and their compilation into the C ABI's
expression table (t3_material).

The Python classes keep Tina's constructors and composition operators
(`a + b`, `a * factor`, `a.mix(b, factor)`).  `compile_material` turns a
material tree into value nodes (CONST / ATTR / INPUT / FRESNEL, children before
parents) followed by the material nodes (LAMBERT, PHONG, COOK, EMISSION, MIX,
SCALE, ADD); the library flattens that tree into weighted lobes for the kernel.
"""
from . import _native as N
from .nodes import ChessboardTexture, Const, FaceAttr, Input, Node, Param, Texture


class IMaterial(Node):
    def __add__(self, other):
        return AddMaterial(self, other)

    def mix(self, other, factor):
        return MixMaterial(self, other, factor)

    def __mul__(self, factor):
        return ScaleMaterial(self, factor)

    def __rmul__(self, factor):
        return ScaleMaterial(self, factor)


class FresnelFactor(Node):
    """f0 = metallic * albedo + (1 - metallic) * 0.16 * specular**2
    (tina/matr/material.py:68-83)."""
    arguments = ['metallic', 'albedo', 'specular']
    defaults = [0.0, 1.0, 0.5]


class MixMaterial(IMaterial):
    """(1 - factor) * mat1 + factor * mat2 (tina/matr/material.py:86-145)."""
    arguments = ['factor']
    defaults = [0.5]

    def __init__(self, mat1, mat2, factor):
        super().__init__(factor=factor)
        self.mat1 = mat1
        self.mat2 = mat2


class ScaleMaterial(IMaterial):
    """factor * mat (tina/matr/material.py:148-191)."""
    arguments = ['factor']
    defaults = [1.0]

    def __init__(self, mat, factor):
        super().__init__(factor=factor)
        self.mat = mat


class AddMaterial(IMaterial):
    """mat1 + mat2 (tina/matr/material.py:194-238)."""
    arguments = []
    defaults = []

    def __init__(self, mat1, mat2):
        super().__init__()
        self.mat1 = mat1
        self.mat2 = mat2


class CookTorrance(IMaterial):
    """GGX-style microfacet lobe (tina/matr/material.py:244-384), reproduced with
    the reference's D = a2 / denom**2 (no 1/pi) and its G normalisation
    1 / lerp(a2, 1, 4*pi)."""
    arguments = ['roughness', 'fresnel']
    defaults = [0.4, 1.0]


class Lambert(IMaterial):
    """brdf = 1/pi (tina/matr/material.py:387-442)."""
    arguments = []
    defaults = []


class Phong(IMaterial):
    """brdf = max(0, V.reflect(-L, n))**m * (m + 2) / 2 (tina/matr/material.py:445-472)."""
    arguments = ['shineness']
    defaults = [32.0]


class Emission(IMaterial):
    """emission = 1, brdf = ambient = 0 (tina/matr/material.py:659-681)."""
    arguments = []
    defaults = []


def Classic(color='color', shineness=32, specular=0.4):
    """(tina/matr/material.py:684-688)"""
    mat_diff = Lambert() * color
    mat_spec = Phong(shineness=shineness)
    return MixMaterial(mat_diff, mat_spec, specular)


def Diffuse(color='color'):
    """(tina/matr/material.py:691-693)"""
    return Lambert() * color


def Lamp(color='color'):
    """(tina/matr/material.py:696-698)"""
    return Emission() * color


def PBR(basecolor='color', metallic=0.0, roughness=0.4, specular=0.5):
    """(tina/matr/material.py:701-706)"""
    mat_diff = Lambert() * basecolor
    f0 = FresnelFactor(metallic=metallic, albedo=basecolor, specular=specular)
    mat_spec = CookTorrance(roughness=roughness, fresnel=f0)
    return MixMaterial(mat_diff, mat_spec, f0)


class MaterialCompileError(ValueError):
    pass


def compile_material(material, attr_stride=0, device=None, keep=None):
    """Returns (t3_material, uses_face_attrs); texture pointers are placed on
    `device` (default: the CUDA device), kept alive through `keep`."""
    nodes = []
    index = {}
    uses_attr = [False]
    textures = []

    def emit(op, a=0, b=0, c=0, v=(0.0, 0.0, 0.0, 0.0)):
        if len(nodes) >= N.T3_MAX_NODES:
            raise MaterialCompileError(f'material needs more than {N.T3_MAX_NODES} nodes')
        nodes.append((op, a, b, c, tuple(v) + (0.0,) * (4 - len(v))))
        return len(nodes) - 1

    def value(node):
        key = id(node)
        if key in index:
            return index[key]
        if isinstance(node, Const) or isinstance(node, Param):
            v = node.value
            if isinstance(v, (tuple, list)):
                vals = tuple(float(x) for x in v)
                if len(vals) == 1:
                    i = emit(N.T3_OP_CONST, 0, 1, 0, (vals[0], vals[0], vals[0], 0.0))
                else:
                    i = emit(N.T3_OP_CONST, 0, 3, 0, vals + (0.0,))
            else:
                is_int = isinstance(node, Const) and node.is_int
                f = float(v)
                i = emit(N.T3_OP_CONST, 0, 1, 1 if is_int else 0, (f, f, f, 0.0))
        elif isinstance(node, Input):
            i = emit(N.T3_OP_INPUT, Input.NAMES[node.name])
        elif isinstance(node, FaceAttr):
            uses_attr[0] = True
            if attr_stride and node.channel + node.width > attr_stride:
                raise MaterialCompileError(
                    f'FaceAttr({node.channel}, {node.width}) exceeds the mesh attribute width {attr_stride}')
            i = emit(N.T3_OP_ATTR, node.channel, node.width)
        elif isinstance(node, FresnelFactor):
            m = value(node.params['metallic'])
            a = value(node.params['albedo'])
            s = value(node.params['specular'])
            i = emit(N.T3_OP_FRESNEL, m, a, s)
        elif isinstance(node, Texture):
            uv = value(node.params['texcoord'])
            if node not in textures:
                if len(textures) >= N.T3_MAX_TEXTURES:
                    raise MaterialCompileError(f'at most {N.T3_MAX_TEXTURES} textures per material')
                textures.append(node)
            i = emit(N.T3_OP_TEXTURE, uv, textures.index(node))
        elif isinstance(node, ChessboardTexture):
            uv = value(node.params['texcoord'])
            size = value(node.params['size'])
            c0 = value(node.params['color0'])
            c1 = value(node.params['color1'])
            i = emit(N.T3_OP_CHECKER, uv, size, c0, (float(c1), 0.0, 0.0, 0.0))
        else:
            raise MaterialCompileError(f'{type(node).__name__} cannot be used as a value')
        index[key] = i
        return i

    def mat(node):
        key = id(node)
        if key in index:
            return index[key]
        if isinstance(node, Lambert):
            i = emit(N.T3_OP_LAMBERT)
        elif isinstance(node, Emission):
            i = emit(N.T3_OP_EMISSION)
        elif isinstance(node, Phong):
            i = emit(N.T3_OP_PHONG, value(node.params['shineness']))
        elif isinstance(node, CookTorrance):
            r = value(node.params['roughness'])
            f = value(node.params['fresnel'])
            i = emit(N.T3_OP_COOK, r, f)
        elif isinstance(node, MixMaterial):
            f = value(node.params['factor'])
            a = mat(node.mat1)
            b = mat(node.mat2)
            i = emit(N.T3_OP_MIX, a, b, f)
        elif isinstance(node, ScaleMaterial):
            f = value(node.params['factor'])
            a = mat(node.mat)
            i = emit(N.T3_OP_SCALE, a, f)
        elif isinstance(node, AddMaterial):
            a = mat(node.mat1)
            b = mat(node.mat2)
            i = emit(N.T3_OP_ADD, a, b)
        else:
            raise MaterialCompileError(
                f'{type(node).__name__} is not supported by the triangle rasteriser build')
        index[key] = i
        return i

    root = mat(material)
    out = N.t3_material()
    out.nnodes = len(nodes)
    out.root = root
    for k, (op, a, b, c, v) in enumerate(nodes):
        nd = out.nodes[k]
        nd.op, nd.a, nd.b, nd.c = op, a, b, c
        for j in range(4):
            nd.v[j] = v[j]
    if textures:
        from ._device import ptr
        keep = keep if keep is not None else []
        for k, t in enumerate(textures):
            out.textures[k].data = ptr(t.data, device or 'cuda', keep)
            out.textures[k].w, out.textures[k].h = t.shape
            out.textures[k].channels = t.channels
    return out, uses_attr[0]
