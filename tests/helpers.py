"""Scene builders shared by the tests."""
import numpy as np

import taichi_three_gb300 as tina


def ndc_from_pixels(px, W, H, z=0.5):
    """World positions whose NDC under W2V = diag(1, 1, -1, 1) land on pixel
    coordinates px ([n, 2]) at depth z."""
    px = np.asarray(px, dtype=np.float64)
    x = px[:, 0] / W * 2 - 1
    y = px[:, 1] / H * 2 - 1
    return np.stack([x, y, -np.full_like(x, z)], axis=1)  # W2V flips z


def flat_scene(tris, W=8, H=8, z=None, material=None, **options):
    """Scene with the default engine matrices (W2V = diag(1,1,-1,1)) and triangles
    given in pixel coordinates: tris [n, 3, 2], z per triangle (default 0.5)."""
    opts = dict(tonemap=False)
    opts.update(options)
    scene = tina.Scene(W, H, **opts)
    tris = np.asarray(tris, dtype=np.float64)
    n = len(tris)
    zs = np.full(n, 0.5) if z is None else np.asarray(z, dtype=np.float64)
    verts = np.stack([ndc_from_pixels(t, W, H, zz) for t, zz in zip(tris, zs)]).astype(np.float32)
    mesh = tina.SimpleMesh()
    mesh.set_face_verts(verts)
    norms = np.zeros_like(verts)
    norms[..., 2] = 1.0
    mesh.set_face_norms(norms)
    scene.add_object(mesh, material or tina.Diffuse(color=1.0))
    return scene, mesh


def random_soup_scene(seed, ntri=300, res=(64, 48), material='pbr', nlights=3, **options):
    """Seeded PBR / Classic soup (moderately large faces) for parity tests."""
    verts, norms, attrs = tina.workloads.soup_arrays(ntri, seed, median_sigma=0.08, log_sd=0.6)
    scene, mesh = tina.workloads.soup_scene(ntri=ntri, res=res, seed=seed, material=material,
                                            nlights=nlights, arrays=(verts, norms, attrs), **options)
    return scene, mesh
