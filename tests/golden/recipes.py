"""Golden scenes, written once against Tina's public API.

Each recipe takes the `tina` module it should use -- the reference package
(executed under the Taichi stand-in by make_golden.py) or taichi_three_gb300 --
plus the scene's seeded input arrays, and builds the scene with identical calls.
That the same code runs on both is the drop-in check; the saved outputs are the
golden vectors.
"""
import numpy as np


def _soup(n, seed, spread=0.9, sigma=0.3):
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(-spread, spread, size=(n, 1, 3))
    verts = (centres + rng.normal(0, sigma, size=(n, 3, 3))).astype(np.float32)
    nrm = rng.normal(size=(n, 3, 3))
    norms = (nrm / np.linalg.norm(nrm, axis=-1, keepdims=True)).astype(np.float32)
    return verts, norms


def inputs(name):
    """Seeded input arrays of each golden scene."""
    if name == 'tri_pair':
        # two faces sharing an edge, given in NDC (default engine matrices)
        v = np.array([[[-1, -1, -0.5], [1, -1, -0.5], [-1, 1, -0.5]],
                      [[1, -1, -0.5], [1, 1, -0.5], [-1, 1, -0.5]],
                      [[-0.6, -0.9, -0.2], [0.7, -0.2, -0.8], [-0.3, 0.8, -0.1]]], np.float32)
        return {'verts': v}
    if name in ('soup_pbr', 'soup_classic', 'soup_transform', 'two_objects'):
        seed = {'soup_pbr': 1, 'soup_classic': 2, 'soup_transform': 3, 'two_objects': 4}[name]
        verts, norms = _soup(240, seed)
        out = {'verts': verts, 'norms': norms}
        if name == 'two_objects':
            v2, n2 = _soup(160, seed + 100)
            out.update(verts2=v2, norms2=n2)
        return out
    if name == 'grid_pbr':
        n = 9
        u = np.linspace(0, 1, n)
        x, y = np.meshgrid(u * 2 - 1, u * 2 - 1, indexing='ij')
        pos = np.stack([x, y, 0.15 * np.sin(3 * x + 0.5) * np.cos(2 * y)], -1).astype(np.float32)
        return {'pos': pos}
    if name == 'sphere_lambert':
        return {}
    if name in ('particles', 'pars_mixed'):
        rng = np.random.Generator(np.random.PCG64(11 if name == 'particles' else 12))
        n = 60
        out = {'pos': rng.uniform(-0.8, 0.8, size=(n, 3)).astype(np.float32),
               'radii': rng.uniform(0.05, 0.24, size=n).astype(np.float32),
               'colors': rng.uniform(0.2, 1.0, size=(n, 3)).astype(np.float32)}
        if name == 'pars_mixed':
            verts, norms = _soup(80, 13, sigma=0.35)
            out.update(verts=verts, norms=norms)
        return out
    if name == 'wire_soup':
        verts, norms = _soup(40, 21, sigma=0.3)
        return {'verts': verts, 'norms': norms}
    if name == 'lines':
        rng = np.random.Generator(np.random.PCG64(22))
        ends = rng.uniform(-1.3, 1.3, size=(70, 2, 3)).astype(np.float32)
        ends[:, :, 2] *= 0.5
        ends[0] = [[-0.5, 0.2, 0.1], [-0.5, 0.2, 0.1]]          # zero length: no step in the frame
        ends[1] = [[0.1, 0.1, 0.0], [0.12, 0.105, 0.0]]         # under a pixel: one step, 0/0 weight
        ends[2] = [[-0.9, -0.4, 0.2], [0.9, -0.4, 0.2]]         # horizontal
        ends[3] = [[0.3, -0.95, -0.1], [0.3, 0.95, 0.3]]        # vertical
        ends[4] = [[-4.0, -3.0, 0.0], [4.0, 2.5, 0.0]]          # both ends far outside the frame
        return {'verts': ends}
    if name == 'wire_grid':
        n = 7
        u = np.linspace(0, 1, n)
        x, y = np.meshgrid(u * 2 - 1, u * 2 - 1, indexing='ij')
        pos = np.stack([x, y, 0.2 * np.cos(2 * x) * np.sin(3 * y + 0.3)], -1).astype(np.float32)
        return {'pos': pos}
    if name == 'wire_quads':
        u = np.linspace(0, 1, 6)
        x, y = np.meshgrid(u * 2 - 1, u * 2 - 1, indexing='ij')
        pos = np.stack([x * 1.1, y * 0.9, 0.25 + 0.15 * np.sin(2 * x + 0.4) * np.cos(3 * y)], -1)
        u2 = np.linspace(0, 1, 9)
        x2, y2 = np.meshgrid(u2 * 2 - 1, u2 * 2 - 1, indexing='ij')
        pos2 = np.stack([x2, y2, 0.1 * np.cos(3 * x2) * np.sin(2 * y2 + 0.2)], -1)
        return {'pos': pos.astype(np.float32), 'pos2': pos2.astype(np.float32)}
    if name == 'textured':
        verts, norms = _soup(60, 31, sigma=0.35)
        rng = np.random.Generator(np.random.PCG64(32))
        coors = rng.uniform(0.03, 0.97, size=(60, 3, 2)).astype(np.float32)
        image = rng.uniform(0.0, 1.0, size=(8, 6, 3)).astype(np.float32)
        v2, n2 = _soup(50, 33, sigma=0.35)
        c2 = rng.uniform(0.03, 0.97, size=(50, 3, 2)).astype(np.float32)
        return {'verts': verts, 'norms': norms, 'coors': coors, 'image': image,
                'verts2': v2, 'norms2': n2, 'coors2': c2}
    if name == 'materials':
        out = {}
        for k in range(6):
            v, n = _soup(40, 71 + k, spread=0.5, sigma=0.3)
            out[f'verts{k}'] = v + np.float32([(k % 3) * 0.7 - 0.7, (k // 3) * 0.8 - 0.4, 0.0])
            out[f'norms{k}'] = n
        return out
    if name == 'mesh_edits':
        verts, norms = _soup(120, 81, spread=0.7, sigma=0.3)
        v2, n2 = _soup(80, 82, spread=0.6, sigma=0.3)
        return {'verts': verts, 'norms': norms, 'verts2': v2, 'norms2': n2}
    if name == 'indexed_ortho':
        v, f = _bumpy_sphere(43, nlat=8, nlon=12)
        n = v / np.linalg.norm(v, axis=1, keepdims=True)
        return {'v': v, 'n': n.astype(np.float32), 'f': f}
    if name == 'smooth_model':
        return {'v': _bumpy_sphere(41)[0], 'f': _bumpy_sphere(41)[1],
                'v2': _bumpy_sphere(42, nlat=6, nlon=9)[0], 'f2': _bumpy_sphere(42, nlat=6, nlon=9)[1]}
    raise KeyError(name)


def _bumpy_sphere(seed, nlat=9, nlon=14):
    """An indexed lat-long sphere with shared, randomly displaced vertices, one
    degenerate face (a repeated vertex) and one vertex no face uses."""
    rng = np.random.Generator(np.random.PCG64(seed))
    v = [[0.0, 0.0, 1.0]]
    for i in range(1, nlat):
        th = np.pi * i / nlat
        for j in range(nlon):
            ph = 2 * np.pi * j / nlon
            v.append([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
    v.append([0.0, 0.0, -1.0])
    v = np.array(v) * rng.uniform(0.85, 1.15, size=(len(v), 1))
    ring = lambda i, j: 1 + (i - 1) * nlon + j % nlon
    f = [[0, ring(1, j), ring(1, j + 1)] for j in range(nlon)]
    for i in range(1, nlat - 1):
        for j in range(nlon):
            f.append([ring(i, j), ring(i + 1, j), ring(i + 1, j + 1)])
            f.append([ring(i, j), ring(i + 1, j + 1), ring(i, j + 1)])
    last = len(v) - 1
    f += [[last, ring(nlat - 1, j + 1), ring(nlat - 1, j)] for j in range(nlon)]
    f.append([ring(2, 0), ring(2, 0), ring(2, 1)])
    v = np.concatenate([v, [[3.0, 3.0, 3.0]]])
    return v.astype(np.float32), np.array(f, np.int32)


def _obj(v, f):
    fi = np.stack([f, np.zeros_like(f), np.zeros_like(f)], axis=2)
    return {'v': v, 'vt': np.zeros((1, 2), np.float32), 'vn': np.zeros((1, 3), np.float32), 'f': fi}


NAMES = ['tri_pair', 'sphere_lambert', 'soup_pbr', 'soup_classic', 'soup_transform', 'grid_pbr',
         'two_objects', 'particles', 'pars_mixed', 'wire_soup', 'lines', 'wire_grid', 'smooth_model',
         'wire_quads', 'textured', 'materials', 'mesh_edits', 'indexed_ortho']


def build(tina, name, arrays, matrix):
    """Builds scene `name` with module `tina`; `matrix` provides lookat/perspective
    (tina.util.matrix in the reference).  Returns (scene, single_object)."""
    if name == 'tri_pair':
        scene = tina.Scene(16, 12)
        mesh = tina.SimpleMesh()
        scene.add_object(mesh)
        mesh.set_face_verts(arrays['verts'])
        return scene, True
    if name == 'sphere_lambert':
        scene = tina.Scene(64, 64, smoothing=True)
        mesh = tina.PrimitiveMesh.sphere(lons=24, lats=12)
        scene.add_object(mesh, tina.Diffuse(color=0.8))
        scene.lighting.clear_lights()
        scene.lighting.add_light(dir=[1, 1, -1])
        scene.lighting.add_light(dir=[0.3, 0.5, 1.0], color=[0.6, 0.5, 0.4])
        scene.lighting.set_ambient_light([0.0, 0.0, 0.0])
        scene.engine.set_camera(matrix.lookat(back=(0, 0, 3)), matrix.perspective(60, 1))
        return scene, True
    if name == 'soup_pbr':
        scene = tina.Scene(48, 36, smoothing=True)
        mesh = tina.SimpleMesh()
        scene.add_object(mesh, tina.PBR(basecolor=[0.8, 0.4, 0.2], metallic=0.3, roughness=0.35))
        mesh.set_face_verts(arrays['verts'])
        mesh.set_face_norms(arrays['norms'])
        scene.lighting.clear_lights()
        scene.lighting.add_light(pos=[1.5, 1.0, 2.0], color=[3.0, 3.0, 3.0])
        scene.lighting.add_light(pos=[-2.0, 0.5, 1.0], color=[1.0, 2.0, 1.5])
        scene.lighting.add_light(dir=[0.2, -0.4, 1.0], color=[0.3, 0.3, 0.3])
        scene.lighting.set_ambient_light([0.05, 0.05, 0.05])
        scene.engine.set_camera(matrix.lookat(back=(0.3, 0.2, 3)), matrix.perspective(60, 48 / 36))
        return scene, True
    if name == 'soup_classic':
        scene = tina.Scene(48, 36, culling=False)
        mesh = tina.SimpleMesh()
        scene.add_object(mesh, tina.Classic())
        mesh.set_face_verts(arrays['verts'])
        scene.engine.set_camera(matrix.lookat(back=(-0.4, 0.3, 3)), matrix.perspective(55, 48 / 36))
        return scene, True
    if name == 'soup_transform':
        scene = tina.Scene(40, 40, smoothing=True, tonemap=False, bgcolor=0.1)
        mesh = tina.SimpleMesh()
        mesh.set_face_verts(arrays['verts'])
        mesh.set_face_norms(arrays['norms'])
        trans = tina.MeshTransform(mesh)
        trans.set_transform(matrix.translate([0.2, -0.1, 0.3]) @ matrix.scale([0.8, 1.2, 0.9]))
        scene.add_object(tina.MeshNoCulling(trans), tina.Diffuse(color=[0.2, 0.7, 0.4]))
        scene.engine.set_camera(matrix.lookat(back=(0, 0, 3)), matrix.perspective(60, 1))
        return scene, True
    if name == 'grid_pbr':
        scene = tina.Scene(48, 36, smoothing=True)
        grid = tina.MeshGrid(9)
        _set_grid(grid, arrays['pos'])
        scene.add_object(grid, tina.PBR(metallic=0.8, roughness=0.5))
        scene.engine.set_camera(matrix.lookat(back=(0.3, -1.2, 2.2)), matrix.perspective(60, 48 / 36))
        return scene, True
    if name == 'two_objects':
        scene = tina.Scene(48, 36, smoothing=True)
        m1 = tina.SimpleMesh()
        m1.set_face_verts(arrays['verts'])
        m1.set_face_norms(arrays['norms'])
        m2 = tina.SimpleMesh()
        m2.set_face_verts(arrays['verts2'])
        m2.set_face_norms(arrays['norms2'])
        scene.add_object(m1, tina.Diffuse(color=[0.9, 0.6, 0.3]))
        scene.add_object(m2, tina.Lamp(color=[0.2, 0.5, 1.0]))
        scene.engine.set_camera(matrix.lookat(back=(0, 0, 3)), matrix.perspective(60, 48 / 36))
        return scene, False
    if name == 'particles':
        scene = tina.Scene(48, 36)
        pars = tina.SimpleParticles(maxpars=64)
        pars.set_particles(arrays['pos'])
        pars.set_particle_radii(arrays['radii'])
        pars.set_particle_colors(arrays['colors'])
        scene.add_object(pars, tina.PBR(basecolor='color', metallic=0.2, roughness=0.4))
        scene.lighting.clear_lights()
        scene.lighting.add_light(pos=[1.5, 1.0, 2.0], color=[3.0, 3.0, 3.0])
        scene.lighting.add_light(dir=[0.2, -0.4, 1.0], color=[0.4, 0.4, 0.4])
        scene.engine.set_camera(matrix.lookat(back=(0.2, 0.3, 3)), matrix.perspective(60, 48 / 36))
        return scene, True
    if name == 'pars_mixed':
        scene = tina.Scene(48, 36, smoothing=True)
        mesh = tina.SimpleMesh()
        mesh.set_face_verts(arrays['verts'])
        mesh.set_face_norms(arrays['norms'])
        scene.add_object(mesh, tina.Diffuse(color=[0.9, 0.6, 0.3]))
        pars = tina.SimpleParticles(maxpars=64)
        pars.set_particles(arrays['pos'])
        pars.set_particle_radii(arrays['radii'])
        pars.set_particle_colors(arrays['colors'])
        scene.add_object(pars, tina.Classic())
        scene.engine.set_camera(matrix.lookat(back=(-0.3, 0.2, 3)), matrix.perspective(60, 48 / 36))
        return scene, False
    if name == 'wire_soup':
        # a mesh's wireframe drawn over the mesh (the reference's wireframe example)
        scene = tina.Scene(48, 36, smoothing=True)
        mesh = tina.SimpleMesh()
        mesh.set_face_verts(arrays['verts'])
        mesh.set_face_norms(arrays['norms'])
        scene.add_object(tina.MeshToWire(mesh))
        inner = tina.MeshTransform(mesh)
        inner.set_transform(matrix.scale([0.9, 0.9, 0.9]))
        scene.add_object(inner, tina.Diffuse(color=[0.4, 0.6, 0.9]))
        scene.engine.set_camera(matrix.lookat(back=(0.2, 0.1, 3)), matrix.perspective(60, 48 / 36))
        return scene, False
    if name == 'lines':
        scene = tina.Scene(40, 30, tonemap=False, bgcolor=0.05, clipping=True,
                           linecolor=(0.2, 0.9, 0.5))
        lines = tina.SimpleMesh(npolygon=2)
        lines.set_face_verts(arrays['verts'])
        scene.add_object(lines)
        scene.engine.set_camera(matrix.lookat(back=(0, 0, 3)), matrix.perspective(60, 40 / 30))
        return scene, False
    if name == 'wire_grid':
        scene = tina.Scene(48, 36, smoothing=True)
        grid = tina.MeshGrid(7)
        _set_grid(grid, arrays['pos'])
        # the wireframe first: where a line and the surface tie in depth the
        # earlier object keeps the pixel
        scene.add_object(tina.MeshToWire(grid))
        scene.add_object(grid, tina.PBR(metallic=0.3, roughness=0.4))
        scene.engine.set_camera(matrix.lookat(back=(0.3, -1.2, 2.2)), matrix.perspective(60, 48 / 36))
        return scene, False
    if name == 'wire_quads':
        # a quad grid's wireframe (four lines per cell) over a triangle grid
        scene = tina.Scene(48, 36, smoothing=True, linecolor=(0.3, 0.8, 1.0))
        quads = tina.MeshGrid(6, as_quad=True)
        _set_grid(quads, arrays['pos'])
        scene.add_object(tina.MeshToWire(quads))
        surface = tina.MeshGrid(9)
        _set_grid(surface, arrays['pos2'])
        scene.add_object(surface, tina.Classic())
        scene.engine.set_camera(matrix.lookat(back=(0.2, -1.0, 2.4)), matrix.perspective(60, 48 / 36))
        return scene, False
    if name == 'textured':
        # an image texture (bilinear at texcoord * (shape - 1)) and a
        # chessboard, both read at interpolated texcoords inside (0, 1)
        scene = tina.Scene(48, 36, smoothing=True, texturing=True)
        mesh = tina.SimpleMesh()
        mesh.set_face_verts(arrays['verts'])
        mesh.set_face_norms(arrays['norms'])
        mesh.set_face_coors(arrays['coors'])
        scene.add_object(mesh, tina.Diffuse(color=tina.Texture(arrays['image'])))
        board = tina.SimpleMesh()
        board.set_face_verts(arrays['verts2'])
        board.set_face_norms(arrays['norms2'])
        board.set_face_coors(arrays['coors2'])
        checker = tina.ChessboardTexture(size=0.2, color0=0.2, color1=[0.9, 0.5, 0.1])
        scene.add_object(board, tina.PBR(basecolor=checker, metallic=0.2, roughness=0.45))
        scene.engine.set_camera(matrix.lookat(back=(0.2, 0.3, 3)), matrix.perspective(60, 48 / 36))
        return scene, False
    if name == 'materials':
        # every material composition: Lambert, Phong, CookTorrance alone, an
        # AddMaterial with Emission, a Mix by an Input, PBR by an Input
        scene = tina.Scene(64, 48, smoothing=True)
        mats = [tina.Lambert(), tina.Phong(shineness=12.5), tina.CookTorrance(roughness=0.3, fresnel=0.5),
                tina.Lambert() * [0.2, 0.4, 0.6] + tina.Emission() * 0.1,
                tina.MixMaterial(tina.Lambert(), tina.Phong(shineness=8), tina.Input('normal')),
                tina.PBR(basecolor=tina.Input('pos'), metallic=0.5, roughness=0.6)]
        for k, mat in enumerate(mats):
            mesh = tina.SimpleMesh()
            mesh.set_face_verts(arrays[f'verts{k}'])
            mesh.set_face_norms(arrays[f'norms{k}'])
            scene.add_object(mesh, mat)
        scene.lighting.set_ambient_light([0.05, 0.1, 0.02])
        scene.lighting.add_light(dir=[0.2, -1, 0.5], color=[0.5, 0.5, 0.5])
        scene.lighting.add_light(pos=[0.5, 0.8, 1.5], color=[0.8, 0.7, 0.6])
        scene.engine.set_camera(matrix.lookat(back=(0.1, 0.2, 3.2)), matrix.perspective(60, 64 / 48))
        return scene, False
    if name == 'mesh_edits':
        # MeshNoCulling(MeshFlipNormal(MeshFlipCulling(MeshTransform(soup)))) and
        # MeshFlatNormal(soup) (tina/mesh/cull.py, norm.py, trans.py)
        scene = tina.Scene(64, 48, smoothing=True)
        base = tina.SimpleMesh()
        base.set_face_verts(arrays['verts'])
        base.set_face_norms(arrays['norms'])
        moved = tina.MeshTransform(base)
        moved.set_transform(matrix.translate([0.3, -0.1, 0.2]) @ matrix.scale([0.7, 1.1, 0.9]))
        scene.add_object(tina.MeshNoCulling(tina.MeshFlipNormal(tina.MeshFlipCulling(moved))),
                         tina.PBR(basecolor=[0.7, 0.5, 0.3], metallic=0.3, roughness=0.35))
        other = tina.SimpleMesh()
        other.set_face_verts(arrays['verts2'])
        other.set_face_norms(arrays['norms2'])
        scene.add_object(tina.MeshFlatNormal(other), tina.Classic(color=[0.9, 0.3, 0.2]))
        scene.engine.set_camera(matrix.lookat(back=(1, 1, 2.5)), matrix.perspective(50, 64 / 48))
        return scene, False
    if name == 'indexed_ortho':
        # an indexed mesh (tina/mesh/conn.py: shared vertices and normals, int
        # face indices) seen through an orthographic projection
        scene = tina.Scene(48, 36, smoothing=True)
        conn = tina.ConnectiveMesh()
        conn.set_vertices(arrays['v'])
        conn.set_vert_norms(arrays['n'])
        conn.set_faces(arrays['f'])
        scene.add_object(conn, tina.PBR(basecolor=[0.5, 0.7, 0.4], metallic=0.1, roughness=0.5))
        scene.engine.set_camera(matrix.lookat(back=(0.5, 0.4, 3)), matrix.orthogonal(1.4, 48 / 36))
        return scene, True
    if name == 'smooth_model':
        scene = tina.Scene(48, 36, smoothing=True)
        model = tina.MeshSmoothNormal(tina.MeshModel(_obj(arrays['v'], arrays['f'])))
        scene.add_object(model, tina.PBR(basecolor=[0.6, 0.7, 0.9], metallic=0.1, roughness=0.3))
        # (the reference's MeshTransform cannot wrap a MeshModel: its getters return tuples)
        v2 = arrays['v2'] * np.float32(0.45) + np.float32([0.9, 0.5, 0.4])
        small = tina.MeshSmoothNormal(tina.MeshModel(_obj(v2.astype(np.float32), arrays['f2'])))
        scene.add_object(small, tina.Classic())
        scene.engine.set_camera(matrix.lookat(back=(0.4, 0.3, 3.2)), matrix.perspective(60, 48 / 36))
        return scene, False
    raise KeyError(name)


def _set_grid(grid, pos):
    p = grid.pos
    if hasattr(p, 'from_numpy'):       # a Taichi field (reference)
        p.from_numpy(pos)
    else:                              # a torch tensor
        import torch
        p.copy_(torch.from_numpy(pos).to(p.device))
