"""Seeded synthetic scenes for the benchmark configurations.

No public dataset is involved: every scene is generated from a numpy PCG64
seed with the shapes and value distributions of the benchmark definitions.

  sphere_scene   512x512 UV sphere (64 lon x 32 lat; Tina's generator yields
                 3,968 faces), Diffuse(0.8), one directional lamp (1, 1, -1).
  soup_scene     1920x1080 triangle soup: T faces with centres U[-1,1]^3,
                 vertices centre + N(0, sigma^2 I), sigma lognormal (median
                 0.004, log-sd 0.7); random unit vertex normals; per-face PBR
                 (roughness U[0.05,1], metallic Bernoulli(0.3), albedo U[0,1]^3)
                 through FaceAttr; 8 point lamps on the radius-3 sphere with
                 intensity U[1,5].
"""
import numpy as np

from . import materials as M
from .matrix import lookat, perspective
from .mesh import PrimitiveMesh, SimpleMesh
from .nodes import FaceAttr
from .scene import Scene


def sphere_scene(res=512, **options):
    opts = dict(smoothing=True)
    opts.update(options)
    scene = Scene(res, **opts)
    mesh = PrimitiveMesh.sphere(lons=64, lats=32, rad=1)
    scene.add_object(mesh, M.Diffuse(color=0.8))
    scene.lighting.clear_lights()
    scene.lighting.add_light(dir=[1, 1, -1])
    scene.lighting.set_ambient_light([0.0, 0.0, 0.0])
    scene.engine.set_camera(lookat(back=(0, 0, 3)), perspective(60, res / res))
    return scene, mesh


def soup_arrays(ntri, seed=0, median_sigma=0.004, log_sd=0.7):
    """(verts [T,3,3], norms [T,3,3], attrs [T,5] = albedo rgb, roughness, metallic)"""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(-1.0, 1.0, size=(ntri, 1, 3))
    sigma = np.exp(rng.normal(np.log(median_sigma), log_sd, size=(ntri, 1, 1)))
    verts = (centres + rng.normal(0.0, 1.0, size=(ntri, 3, 3)) * sigma).astype(np.float32)
    n = rng.normal(0.0, 1.0, size=(ntri, 3, 3))
    norms = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    attrs = np.empty((ntri, 5), np.float32)
    attrs[:, 0:3] = rng.uniform(0.0, 1.0, size=(ntri, 3))
    attrs[:, 3] = rng.uniform(0.05, 1.0, size=ntri)
    attrs[:, 4] = (rng.uniform(0.0, 1.0, size=ntri) < 0.3).astype(np.float32)
    return verts, norms, attrs


def point_lights(n=8, seed=0, radius=3.0):
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    d = rng.normal(size=(n, 3))
    d = d / np.linalg.norm(d, axis=-1, keepdims=True) * radius
    inten = rng.uniform(1.0, 5.0, size=n)
    return d, inten


def pbr_face_material():
    """PBR with per-face albedo (channels 0-2), roughness (3), metallic (4)."""
    return M.PBR(basecolor=FaceAttr(0, 3), metallic=FaceAttr(4), roughness=FaceAttr(3))


def classic_face_material():
    """Classic (Lambert + Phong) with per-face albedo."""
    return M.Classic(color=FaceAttr(0, 3))


def soup_scene(ntri=1_000_000, res=(1920, 1080), seed=0, material='pbr', nlights=8, arrays=None,
               **options):
    opts = dict(smoothing=True)
    opts.update(options)
    scene = Scene(res[0], res[1], **opts)
    verts, norms, attrs = arrays if arrays is not None else soup_arrays(ntri, seed)
    mesh = SimpleMesh(maxfaces=max(ntri, 1))
    mesh.set_face_verts(verts)
    mesh.set_face_norms(norms)
    mesh.set_face_attrs(attrs)
    mat = {'pbr': pbr_face_material, 'classic': classic_face_material}[material]()
    scene.add_object(mesh, mat)
    scene.lighting.clear_lights()
    pos, inten = point_lights(nlights, seed)
    for p, i in zip(pos, inten):
        scene.lighting.add_light(pos=p.tolist(), color=[float(i)] * 3)
    scene.lighting.set_ambient_light([0.0, 0.0, 0.0])
    scene.engine.set_camera(lookat(back=(0, 0, 3)), perspective(60, res[0] / res[1]))
    return scene, mesh


def ibl_soup_scene(ntri=1_000_000, res=(1920, 1080), seed=0, env_res=512, mode='mc', spp=256,
                   mlp=None, skybox=None, nlights=0, **options):
    """The soup of soup_scene lit by a procedural equirect environment
    ((2*env_res) x env_res FP16: sky gradient + 12 Gaussian lobes) through
    SkyboxLighting, Monte Carlo (mode 'mc', spp samples) or the learned
    network (mode 'mlp'); nlights point lamps on top (0 by default)."""
    from .skybox import Skybox, SkyboxLighting, procedural_sky
    sky = skybox if skybox is not None else Skybox(procedural_sky(env_res, seed=seed))
    light = SkyboxLighting(sky, mode=mode, spp=spp, seed=seed, mlp=mlp)
    scene, mesh = soup_scene(ntri=ntri, res=res, seed=seed, nlights=0, ibl=True, lighting=light,
                             **options)
    if nlights:
        pos, inten = point_lights(nlights, seed)
        for p, i in zip(pos, inten):
            light.add_light(pos=p.tolist(), color=[float(i)] * 3)
    return scene, mesh


def batch_scenes(n=64, seed=0, t_min=1_000, t_max=2_000_000, resolutions=(256, 512, 768, 1024),
                 nlights=8, material='classic'):
    """Multi-view batch: n soups with T_i = round(exp(U[ln t_min, ln t_max]))
    faces from the soup generator (seed + i), square resolution drawn from
    `resolutions`, camera uniform on the radius-3 sphere looking at the origin,
    Classic (Lambert + Phong) per-face albedo, nlights point lamps."""
    rng = np.random.Generator(np.random.PCG64(seed))
    scenes = []
    for i in range(n):
        T = int(round(np.exp(rng.uniform(np.log(t_min), np.log(t_max)))))
        res = int(rng.choice(resolutions))
        d = rng.normal(size=3)
        d = d / np.linalg.norm(d) * 3.0
        up = (0, 1, 1e-12) if abs(d[1]) < 2.9 else (1, 0, 1e-12)
        scene, _ = soup_scene(ntri=T, res=(res, res), seed=seed * 1000 + i, material=material,
                              nlights=nlights)
        scene.engine.set_camera(lookat(back=tuple(d), up=up), perspective(60, 1.0))
        scenes.append(scene)
    return scenes


def wave_grid_scene(grid_res=2048, res=(3840, 2160), skybox=None, mlp=None, nlights=2, seed=0,
                    lamps_only=False, **options):
    """Animated grid: MeshGrid(grid_res) over [-1, 1]^2 (displaced per frame by
    MeshGrid.displace_wave: z = 0.1 sin(8x + t) cos(8y + 1.3t)), smooth normals,
    PBR (albedo (0.75, 0.62, 0.5), metallic 0.3, roughness 0.35), lit by the
    environment -- the learned network when `mlp` is given, else 256-sample
    Monte Carlo -- plus nlights point lamps; camera in front of and above the
    grid, fov 60.  lamps_only: the same scene lit by its point lamps alone
    (no environment, no ambient)."""
    from .lighting import Lighting
    from .mesh import MeshGrid
    from .skybox import Skybox, SkyboxLighting, procedural_sky
    if lamps_only:
        light = Lighting()
        opts = dict(smoothing=True, lighting=light)
    else:
        sky = skybox if skybox is not None else Skybox(procedural_sky(512, seed=seed))
        light = SkyboxLighting(sky, mode='mlp' if mlp is not None else 'mc', mlp=mlp, spp=256, seed=seed)
        opts = dict(smoothing=True, ibl=True, lighting=light)
    opts.update(options)
    scene = Scene(res[0], res[1], **opts)
    if lamps_only:
        scene.lighting = light
        light.set_ambient_light([0.0, 0.0, 0.0])
    grid = MeshGrid(grid_res)
    scene.add_object(grid, M.PBR(basecolor=(0.75, 0.62, 0.5), metallic=0.3, roughness=0.35))
    pos, inten = point_lights(nlights, seed)
    for p, i in zip(pos, inten):
        light.add_light(pos=p.tolist(), color=[float(i)] * 3)
    scene.engine.set_camera(lookat(back=(0.0, -1.1, 1.45)), perspective(60, res[0] / res[1]))
    return scene, grid
