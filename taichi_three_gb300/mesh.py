"""Mesh nodes: the mesh protocol of Tina's tina/mesh package.

Every mesh fills a t3_mesh descriptor (`_t3_fill`) that the CUDA kernels read
through the same getters the reference calls per face (get_face_verts /
get_face_norms / get_face_coors).  Mesh-edit nodes become descriptor flags and
apply in one fixed nesting,
    MeshNoCulling(MeshFlipNormal(MeshFlipCulling(MeshFlatNormal(MeshTransform(base))))),
any sub-sequence of which may be used; other nestings raise NotImplementedError.
"""
import numpy as np
import torch

from . import _native as N
from ._device import as_f32, as_i32, default_device, ptr

MAX = 2**20  # tina/common.py:7


def _copy_in_place(dst, src, limit=None):
    """Updates the device buffer `dst` from a float32 CPU tensor of the same
    shape (the first `limit` rows): one stream-ordered copy, asynchronous from
    pinned memory, no allocation (Taichi's field.from_numpy also writes the
    field in place).  Returns False when the shapes differ."""
    if dst is None or not isinstance(src, torch.Tensor) or src.device.type != 'cpu':
        return False
    if src.dtype != torch.float32 or not src.is_contiguous():
        return False
    n = src.shape[0] if limit is None else min(src.shape[0], limit)
    if tuple(dst.shape) != (n,) + tuple(src.shape[1:]) or not dst.is_cuda:
        return False
    dst.copy_(src[:n], non_blocking=src.is_pinned())
    return True


class MeshBase:
    face_attr = None

    def get_npolygon(self):
        return 3

    def pre_compute(self):
        pass

    def set_face_attrs(self, attrs):
        """Extension: per-face material attributes [nfaces, C] read by FaceAttr."""
        if _copy_in_place(self.face_attr, attrs):
            return
        a = as_f32(attrs)
        if a.dim() == 1:
            a = a[:, None]
        self.face_attr = a.contiguous()

    def _fill_attr(self, m, device, keep):
        if self.face_attr is not None:
            m.face_attr = ptr(self.face_attr, device, keep)
            m.attr_stride = int(self.face_attr.shape[1])

    def attr_stride(self):
        return 0 if self.face_attr is None else int(self.face_attr.shape[1])


class SimpleMesh(MeshBase):
    """A face soup (tina/mesh/simple.py): verts [n, p, 3], norms [n, p, 3],
    coors [n, p, 2] with p = npolygon, 3 (triangles) or 2 (lines, drawn by the
    wireframe rasteriser); nfaces = min(n, maxfaces)."""

    def __init__(self, maxfaces=MAX, npolygon=3):
        if npolygon not in (2, 3):
            raise NotImplementedError('SimpleMesh takes npolygon=3 (triangles) or 2 (lines) in this build')
        self.maxfaces = maxfaces
        self.npolygon = npolygon
        self.nfaces = 0
        dev = default_device()
        self.verts = torch.zeros((0, npolygon, 3), dtype=torch.float32, device=dev)
        self.norms = None
        self.coors = None

    def get_npolygon(self):
        return self.npolygon

    def get_nfaces(self):
        return min(self.nfaces, self.maxfaces)

    def set_face_verts(self, verts):
        if _copy_in_place(self.verts, verts, self.maxfaces):
            self.nfaces = self.verts.shape[0]
            return
        p = self.npolygon
        v = as_f32(verts)
        if v.dim() != 3 or v.shape[1] != p or v.shape[2] != 3:
            raise ValueError(f'verts must have shape [nfaces, {p}, 3]')
        self.nfaces = min(v.shape[0], self.maxfaces)
        self.verts = v[:self.nfaces].contiguous()

    def set_face_norms(self, norms):
        if self.norms is not None and self.norms.shape[0] == self.nfaces and \
                _copy_in_place(self.norms, norms, self.nfaces):
            return
        p = self.npolygon
        n = as_f32(norms)
        if n.dim() != 3 or n.shape[0] < self.nfaces or n.shape[1:] != (p, 3):
            raise ValueError(f'norms must have shape [>= nfaces, {p}, 3]')
        self.norms = n[:self.nfaces].contiguous()

    def set_face_coors(self, coors):
        if self.coors is not None and self.coors.shape[0] == self.nfaces and \
                _copy_in_place(self.coors, coors, self.nfaces):
            return
        p = self.npolygon
        c = as_f32(coors)
        if c.dim() != 3 or c.shape[0] < self.nfaces or c.shape[1] != p or c.shape[2] < 2:
            raise ValueError(f'coors must have shape [>= nfaces, {p}, 2]')
        self.coors = c[:self.nfaces, :, :2].contiguous()

    def _t3_fill(self, m, device, keep):
        m.kind = N.T3_MESH_SOUP if self.npolygon == 3 else N.T3_MESH_LINES
        m.nfaces = self.get_nfaces()
        m.verts = ptr(self.verts, device, keep)
        m.norms = ptr(self.norms, device, keep)
        m.coors = ptr(self.coors, device, keep)
        self._fill_attr(m, device, keep)


class PrimitiveMesh(SimpleMesh):
    """SimpleMesh built from [n, 3, 3(vert, norm, coor), 3] faces
    (tina/mesh/prim.py:6-26)."""

    def __init__(self, faces):
        faces = np.asarray(faces, dtype=np.float32)
        super().__init__(maxfaces=len(faces), npolygon=faces.shape[1])
        self.set_face_verts(faces[:, :, 0])
        self.set_face_norms(faces[:, :, 1])
        self.set_face_coors(faces[:, :, 2, :2])

    @staticmethod
    def _ring_faces(corner, rows, cols, keep_first=True, keep_last=True):
        """Two triangles (a, b, c) and (c, d, a) per cell of a (rows x cols)
        corner table, a = (i, j), b = (i, j+1), c = (i+1, j+1), d = (i+1, j),
        cells in row-major order; `keep_first` / `keep_last` drop the first
        triangle of the first row and the second of the last row (a sphere's
        poles)."""
        faces = []
        for i in range(rows):
            for j in range(cols):
                a, b, c, d = corner[i][j], corner[i][j + 1], corner[i + 1][j + 1], corner[i + 1][j]
                if keep_first or i != 0:
                    faces.append([a, b, c])
                if keep_last or i != rows - 1:
                    faces.append([c, d, a])
        return faces

    @classmethod
    def sphere(cls, lons=32, lats=24, rad=1):
        """UV sphere with the face order of tina/mesh/prim.py:22-48 (face ids
        must match): corner (i, j) sits at latitude (i / lats - 0.5) pi and
        longitude (2 j / lons - 1) pi with texcoord (j / lons, i / lats); the
        pole rows keep one triangle per cell, so lons=64, lats=32 gives 3,968
        faces."""
        corner = []
        for i in range(lats + 1):
            row = []
            for j in range(lons + 1):
                u, v = j / lons, i / lats
                th, ph = (v - 0.5) * np.pi, (u * 2 - 1) * np.pi
                n = (np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), np.sin(th))
                row.append(((n[0] * rad, n[1] * rad, n[2] * rad), n, (u, v, 0)))
            corner.append(row)
        return cls(cls._ring_faces(corner, lats, lons, keep_first=False, keep_last=False))

    @classmethod
    def cylinder(cls, lons=32, lats=4, rad=1, hei=2):
        """Capped cylinder with the face order of tina/mesh/prim.py:50-88: the
        side cells, then the bottom cap's fan, then the top cap's; corner
        (i, j) at height (i / lats - 0.5) hei and angle (2 j / lons - 1) pi."""
        corner = []
        for i in range(lats + 1):
            row = []
            for j in range(lons + 1):
                u, v = j / lons, i / lats
                ph = (u * 2 - 1) * np.pi
                x, y = np.cos(ph), np.sin(ph)
                row.append(((x * rad, y * rad, (v - 0.5) * hei), (x, y, 0), (u, v, 0)))
            corner.append(row)
        faces = cls._ring_faces(corner, lats, lons)
        down, up = ((0, 0, -1), (0, 0, -1)), ((0, 0, 1), (0, 0, 1))  # (normal, texcoord) of the caps
        for j in range(lons):
            faces.append([(corner[0][j + 1][0],) + down, (corner[0][j][0],) + down, ((0, 0, -hei / 2),) + down])
        for j in range(lons):
            faces.append([((0, 0, hei / 2),) + up, (corner[lats][j][0],) + up, (corner[lats][j + 1][0],) + up])
        return cls(faces)


class MeshGrid(MeshBase):
    """Parametric grid (tina/mesh/grid.py): pos/nrm/tex [nx, ny, 3|2]; two
    triangles per cell (cell m = (m // (ny - 1), m % (ny - 1)): the reference's
    order on square grids, where its stride res.x - 1 equals ny - 1; on a
    rectangular grid that stride would index past the second axis), or with `as_quad=True` one quad per cell (drawn only
    through MeshToWire: four lines per quad); `pre_compute` (run by every
    render) recomputes the smooth normals on the device."""

    def __init__(self, res, as_quad=False):
        self.as_quad = bool(as_quad)
        if isinstance(res, int):
            res = res, res
        self.res = tuple(int(r) for r in res)
        if min(self.res) < 2:
            raise ValueError('MeshGrid needs at least 2 x 2 vertices')
        dev = default_device()
        nx, ny = self.res
        # init_pos (tina/mesh/grid.py:15-20)
        I = torch.stack(torch.meshgrid(torch.arange(nx, dtype=torch.float32),
                                       torch.arange(ny, dtype=torch.float32), indexing='ij'), -1)
        uv = I / torch.tensor([nx - 1, ny - 1], dtype=torch.float32)
        self.tex = uv.to(dev).contiguous()
        pos = torch.zeros((nx, ny, 3), dtype=torch.float32)
        pos[..., 0] = uv[..., 0] * 2 - 1
        pos[..., 1] = uv[..., 1] * 2 - 1
        self.pos = pos.to(dev).contiguous()
        self.nrm = torch.zeros((nx, ny, 3), dtype=torch.float32, device=dev)
        self.auto_normals = True

    def get_npolygon(self):
        return 4 if self.as_quad else 3

    def get_nfaces(self):
        n = (self.res[0] - 1) * (self.res[1] - 1)
        return n if self.as_quad else n * 2

    def displace_wave(self, t, amp=0.1, fx=8.0, fy=8.0, wx=1.0, wy=1.3):
        """pos.z = amp sin(fx x + wx t) cos(fy y + wy t) on the device (the
        animated grid of the benchmark; x, y are the vertices' own)."""
        lib = N.load()
        stream = torch.cuda.current_stream(self.pos.device).cuda_stream
        N.check(lib.t3_grid_wave(self.pos.data_ptr(), self.res[0], self.res[1], amp, fx, fy, wx, wy,
                                 float(t), stream), 't3_grid_wave')

    def pre_compute(self):
        if not self.auto_normals:
            return
        if self.pos.is_cuda:
            lib = N.load()
            stream = torch.cuda.current_stream(self.pos.device).cuda_stream
            N.check(lib.t3_grid_normals(self.pos.data_ptr(), self.nrm.data_ptr(), self.res[0],
                                        self.res[1], stream), 't3_grid_normals')

    def _t3_fill(self, m, device, keep):
        m.kind = N.T3_MESH_GRID
        m.nfaces = self.get_nfaces()
        m.verts = ptr(self.pos, device, keep)
        m.norms = ptr(self.nrm, device, keep)
        m.coors = ptr(self.tex, device, keep)
        m.grid_nx, m.grid_ny = self.res
        if self.as_quad:
            m.flags |= N.T3_MESH_QUADS
        self._fill_attr(m, device, keep)


class ConnectiveMesh(MeshBase):
    """Indexed mesh with shared vertex attributes (tina/mesh/conn.py)."""

    def __init__(self, maxfaces=MAX, maxverts=MAX, npolygon=3):
        if npolygon != 3:
            raise NotImplementedError('only triangle meshes are rasterised by this build')
        self.maxfaces, self.maxverts, self.npolygon = maxfaces, maxverts, npolygon
        dev = default_device()
        self.faces = torch.zeros((0, 3), dtype=torch.int32, device=dev)
        self.verts = torch.zeros((0, 3), dtype=torch.float32, device=dev)
        self.norms = None
        self.coors = None
        self.nfaces = 0

    def get_max_vert_nindex(self):
        return self.maxverts

    def get_nfaces(self):
        return self.nfaces

    def set_vertices(self, verts):
        self.verts = as_f32(verts)[:self.maxverts].contiguous()

    def set_vert_norms(self, norms):
        self.norms = as_f32(norms)[:self.maxverts].contiguous()

    def set_vert_coors(self, coors):
        self.coors = as_f32(coors)[:self.maxverts, :2].contiguous()

    def set_faces(self, faces):
        f = as_i32(faces)
        if f.dim() != 2 or f.shape[1] != 3:
            raise ValueError('faces must have shape [nfaces, 3]')
        self.nfaces = min(f.shape[0], self.maxfaces)
        self.faces = f[:self.nfaces].contiguous()

    def _check_indices(self):
        if self.nfaces == 0:
            return
        lo, hi = int(self.faces.min()), int(self.faces.max())
        for name, arr in (('verts', self.verts), ('norms', self.norms), ('coors', self.coors)):
            if arr is not None and (lo < 0 or hi >= arr.shape[0]):
                raise ValueError(f'face indices [{lo}, {hi}] out of range for {name} ({arr.shape[0]})')

    def _t3_fill(self, m, device, keep):
        self._check_indices()
        m.kind = N.T3_MESH_INDEXED
        m.nfaces = self.nfaces
        m.verts = ptr(self.verts, device, keep)
        m.nverts = int(self.verts.shape[0])
        m.norms = ptr(self.norms, device, keep)
        m.coors = ptr(self.coors, device, keep)
        m.faces = ptr(self.faces, device, keep)
        m.face_stride, m.corner_stride = 3, 1
        m.slot_vert = m.slot_coor = m.slot_norm = 0
        self._fill_attr(m, device, keep)


class MeshModel(MeshBase):
    """Indexed mesh with per-corner (v, vt, vn) indices (tina/mesh/model.py);
    `obj` is a dict with 'v' [nv,3], 'vt' [nt,2], 'vn' [nn,3], 'f' [n,3,3] or [n,3]."""

    def __init__(self, obj):
        if isinstance(obj, str):
            from .assimp import readobj
            obj = readobj(obj)
        f = np.asarray(obj['f'])
        if f.ndim == 2:
            f = np.stack([f, f, f], axis=2)
        self.faces = as_i32(f.reshape(len(f), 9))
        self.verts = as_f32(obj['v'])
        self.coors = as_f32(np.asarray(obj['vt'])[:, :2]) if len(obj.get('vt', [])) else None
        self.norms = as_f32(obj['vn']) if len(obj.get('vn', [])) else None
        self.nfaces = len(f)

    def get_nfaces(self):
        return self.nfaces

    def get_max_vert_nindex(self):
        return int(self.verts.shape[0])

    def _check_indices(self):
        if self.nfaces == 0:
            return
        f = self.faces.view(-1, 3, 3)
        for slot, arr, name in ((0, self.verts, 'v'), (1, self.coors, 'vt'), (2, self.norms, 'vn')):
            if arr is None:
                continue
            lo, hi = int(f[:, :, slot].min()), int(f[:, :, slot].max())
            if lo < 0 or hi >= arr.shape[0]:
                raise ValueError(f'{name} indices [{lo}, {hi}] out of range ({arr.shape[0]})')

    def _t3_fill(self, m, device, keep):
        self._check_indices()
        m.kind = N.T3_MESH_INDEXED
        m.nfaces = self.nfaces
        m.verts = ptr(self.verts, device, keep)
        m.nverts = int(self.verts.shape[0])
        m.norms = ptr(self.norms, device, keep)
        m.coors = ptr(self.coors, device, keep)
        m.faces = ptr(self.faces, device, keep)
        m.face_stride, m.corner_stride = 9, 3
        m.slot_vert, m.slot_coor, m.slot_norm = 0, 1, 2
        self._fill_attr(m, device, keep)


class MeshEditBase:
    """Wraps a mesh and forwards every other attribute (tina/mesh/base.py)."""
    _flag = 0

    def __init__(self, mesh):
        self.mesh = mesh

    def __getattr__(self, attr):
        return getattr(self.mesh, attr)

    def get_nfaces(self):
        return self.mesh.get_nfaces()

    def pre_compute(self):
        self.mesh.pre_compute()

    def _check_inner(self, m, forbidden):
        # T3_MESH_QUADS describes the base grid, not an edit (the library
        # checks which edits may wrap it)
        if m.flags & forbidden & ~N.T3_MESH_QUADS:
            raise NotImplementedError(
                f'{type(self).__name__} around this mesh-edit chain is not supported; nest edits as '
                'MeshNoCulling(MeshFlipNormal(MeshFlipCulling(MeshFlatNormal(MeshTransform(mesh)))))')


class MeshTransform(MeshEditBase):
    """4x4 transform of the vertices and transpose(inv(trans))[:3, :3] of the
    normals (tina/mesh/trans.py:5-40)."""

    def __init__(self, mesh, trans=None):
        super().__init__(mesh)
        self.trans = np.eye(4, dtype=np.float32)
        self.trans_normal = np.eye(3, dtype=np.float32)
        if trans is not None:
            self.set_transform(trans)

    def set_transform(self, trans):
        trans = np.asarray(trans, dtype=np.float64)
        trans_normal = np.transpose(np.linalg.inv(trans))
        self.trans = np.array(trans, dtype=np.float32)
        self.trans_normal = np.array(trans_normal[:3, :3], dtype=np.float32)

    def _t3_fill(self, m, device, keep):
        self.mesh._t3_fill(m, device, keep)
        # a transform commutes with MeshToWire (both act per vertex)
        self._check_inner(m, 0xFF & ~N.T3_MESH_WIREFRAME)
        m.flags |= N.T3_MESH_TRANSFORM
        t = self.trans.reshape(-1)
        tn = self.trans_normal.reshape(-1)
        for k in range(16):
            m.trans[k] = float(t[k])
        for k in range(9):
            m.trans_normal[k] = float(tn[k])


class MeshFlatNormal(MeshEditBase):
    """normals = normalize(cross(b - a, c - a)) per face (tina/mesh/norm.py:5-14)."""

    def _t3_fill(self, m, device, keep):
        self.mesh._t3_fill(m, device, keep)
        self._check_inner(m, N.T3_MESH_FLAT_NORMAL | N.T3_MESH_FLIP_ORDER | N.T3_MESH_FLIP_NORMAL
                          | N.T3_MESH_NOCULL | N.T3_MESH_WIREFRAME)
        m.flags |= N.T3_MESH_FLAT_NORMAL


class MeshFlipCulling(MeshEditBase):
    """Reversed corner order (tina/mesh/cull.py:5-28)."""

    def _t3_fill(self, m, device, keep):
        self.mesh._t3_fill(m, device, keep)
        self._check_inner(m, N.T3_MESH_FLIP_NORMAL | N.T3_MESH_NOCULL | N.T3_MESH_WIREFRAME)
        m.flags ^= N.T3_MESH_FLIP_ORDER


class MeshFlipNormal(MeshEditBase):
    """Negated normals (tina/mesh/cull.py:61-66)."""

    def _t3_fill(self, m, device, keep):
        self.mesh._t3_fill(m, device, keep)
        self._check_inner(m, N.T3_MESH_NOCULL | N.T3_MESH_WIREFRAME)
        m.flags ^= N.T3_MESH_FLIP_NORMAL


class MeshNoCulling(MeshEditBase):
    """Every face twice, odd copies flipped with negated normals
    (tina/mesh/cull.py:31-58)."""

    def get_nfaces(self):
        return self.mesh.get_nfaces() * 2

    def _t3_fill(self, m, device, keep):
        self.mesh._t3_fill(m, device, keep)
        self._check_inner(m, N.T3_MESH_NOCULL | N.T3_MESH_WIREFRAME)
        m.flags |= N.T3_MESH_NOCULL


class MeshSmoothNormal(MeshEditBase):
    """Per-vertex normals of an indexed mesh (tina/mesh/norm.py:17-55): each
    face's unit normal is summed onto its three vertices in face order, the sums
    normalised, and every face corner reads its vertex's normal.  cached=True
    computes them once (at the first render, or by update_normal()),
    cached=False at every pre_compute.  Wraps a ConnectiveMesh or MeshModel
    directly; other edits go outside it."""

    def __init__(self, mesh, cached=True):
        super().__init__(mesh)
        if not isinstance(mesh, (ConnectiveMesh, MeshModel)):
            raise NotImplementedError('MeshSmoothNormal wraps a ConnectiveMesh or MeshModel in this build')
        self.cached = cached
        self.norm = None

    def pre_compute(self):
        self.mesh.pre_compute()
        if not self.cached or self.norm is None:
            self.update_normal()

    def update_normal(self):
        """Recomputes the vertex normals from the current vertices (t3_smooth_normals)."""
        import ctypes as C
        from ._device import require_cuda
        require_cuda('MeshSmoothNormal')
        lib = N.load()
        dev = default_device()
        m = N.t3_mesh()
        keep = []
        self.mesh._t3_fill(m, dev, keep)
        nverts = int(self.mesh.verts.shape[0])
        if self.norm is None or tuple(self.norm.shape) != (nverts, 3) or not self.norm.is_cuda:
            self.norm = torch.empty((nverts, 3), dtype=torch.float32, device=dev)
        size = C.c_size_t()
        N.check(lib.t3_smooth_normals_workspace_size(m.nfaces, nverts, C.byref(size)),
                't3_smooth_normals_workspace_size')
        ws = torch.empty(max(size.value, 16), dtype=torch.uint8, device=dev)
        N.check(lib.t3_smooth_normals(C.byref(m), nverts, self.norm.data_ptr(), ws.data_ptr(), ws.numel(),
                                      torch.cuda.current_stream().cuda_stream), 't3_smooth_normals')

    def _t3_fill(self, m, device, keep):
        self.mesh._t3_fill(m, device, keep)
        if self.norm is None:
            raise RuntimeError('MeshSmoothNormal: normals not computed yet (pre_compute or update_normal)')
        m.norms = ptr(self.norm, device, keep)
        m.slot_norm = m.slot_vert


class MeshToWire(MeshEditBase):
    """The polygon edges of a mesh as lines for the wireframe rasteriser
    (tina/mesh/wire.py:5-40): line n joins corners n % p and (n + 1) % p of
    face n // p, p the wrapped mesh's npolygon; applies outside every other
    edit except MeshTransform."""

    def __init__(self, mesh):
        super().__init__(mesh)
        self.src_npolygon = mesh.get_npolygon() if hasattr(mesh, 'get_npolygon') else 3

    def get_npolygon(self):
        return 2

    def get_nfaces(self):
        return self.mesh.get_nfaces() * self.src_npolygon

    def _t3_fill(self, m, device, keep):
        self.mesh._t3_fill(m, device, keep)
        self._check_inner(m, N.T3_MESH_WIREFRAME)
        m.flags |= N.T3_MESH_WIREFRAME


class SimpleParticles:
    """Particles (tina/pars/simple.py): positions [n, 3], radii [n] (default
    `radius`), colours [n, 3] (default white), rasterised as shaded spheres by
    the particle rasteriser (tina/core/particle.py); Input('color') of the
    material reads the particle's colour."""

    def __init__(self, maxpars=65536, radius=0.02):
        dev = default_device()
        self.maxpars = int(maxpars)
        self.radius = float(radius)
        self.npars = 0
        self.verts = torch.zeros((0, 3), dtype=torch.float32, device=dev)
        self.sizes = torch.zeros((0,), dtype=torch.float32, device=dev)
        self.colors = torch.zeros((0, 3), dtype=torch.float32, device=dev)

    def get_npars(self):
        return min(self.npars, self.maxpars)

    def pre_compute(self):
        pass

    def set_particles(self, verts):
        v = as_f32(verts)
        if v.dim() != 2 or v.shape[1] != 3:
            raise ValueError('particle positions must have shape [n, 3]')
        n = min(v.shape[0], self.maxpars)
        self.npars = n
        self.verts = v[:n].contiguous()
        if self.sizes.shape[0] != n:
            self.sizes = torch.full((n,), self.radius, dtype=torch.float32, device=self.verts.device)
        if self.colors.shape[0] != n:
            self.colors = torch.ones((n, 3), dtype=torch.float32, device=self.verts.device)

    def set_particle_radii(self, sizes):
        s = as_f32(sizes).reshape(-1)
        if s.shape[0] < self.npars:
            raise ValueError('need one radius per particle')
        self.sizes = s[:self.npars].contiguous()

    def set_particle_colors(self, colors):
        c = as_f32(colors)
        if c.dim() != 2 or c.shape[0] < self.npars or c.shape[1] != 3:
            raise ValueError('particle colours must have shape [n, 3]')
        self.colors = c[:self.npars].contiguous()

    def attr_stride(self):
        return 0

    def _t3_fill(self, m, device, keep):
        m.kind = N.T3_MESH_PARTICLES
        m.nfaces = self.get_npars()
        m.verts = ptr(self.verts, device, keep)
        m.coors = ptr(self.sizes, device, keep)
        m.norms = ptr(self.colors, device, keep)
