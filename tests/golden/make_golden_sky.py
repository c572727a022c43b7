"""Generates tests/golden/sky_golden.npz from the reference's own background
pass: tina/core/engine.py Engine.render_background (the view ray of every
empty pixel) with tina/core/shader.py BackgroundShader over a lighting whose
background is tina/skybox.py Skybox.sample (spheremap + bilerp of an
equirectangular map), run under the Taichi stand-in like
make_golden.py.  (The reference's SkyboxLighting would also bake prefiltered
IBL tables from an image asset; the background needs only the skybox.)

Usage:  TINA_REFERENCE=/path/to/taichi_three python tests/golden/make_golden_sky.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

RES = (40, 30)
CAMERAS = {'front': dict(back=(0.3, 0.2, 3.0), fov=60), 'up': dict(back=(0.5, -2.5, 1.0), fov=75)}


def env_map():
    """Seeded HDR equirect map (2*16, 16, 3) with smooth and sharp structure."""
    rng = np.random.Generator(np.random.PCG64(61))
    i, j = np.meshgrid(np.arange(32), np.arange(16), indexing='ij')
    base = 0.5 + 0.4 * np.stack([np.sin(i / 5.0), np.cos(j / 3.0), np.sin((i + j) / 7.0)], -1)
    return (base * rng.uniform(0.5, 2.0, size=(32, 16, 3))).astype(np.float32)


def main():
    import make_golden
    tina, matrix = make_golden.load_reference()
    import taichi_standin as ti
    import importlib
    importlib.import_module('tina.skybox')
    env = env_map()
    out = {'in_env': env}
    for name, cam in CAMERAS.items():
        engine = tina.Engine(RES)
        engine.set_camera(matrix.lookat(back=cam['back']), matrix.perspective(cam['fov'], RES[0] / RES[1]))
        # Skybox(shape) then the texels: the array constructor's fill runs as a
        # materialize callback, which Taichi defers and the stand-in does not
        sky = sys.modules['tina.skybox'].Skybox(env.shape[:2])
        sky.img.from_numpy(env)

        @ti.data_oriented
        class SkyOnly:
            @ti.func
            def background(self, rd):
                return sky.sample(rd)

        img = ti.Vector.field(3, float, RES)
        engine.render_background(tina.BackgroundShader(img, SkyOnly()))
        out['out_' + name] = img.to_numpy().astype(np.float32)
        print(f'{name}: mean {out["out_" + name].mean():.4f}', flush=True)
    np.savez_compressed(os.path.join(HERE, 'sky_golden.npz'), **out)


if __name__ == '__main__':
    main()
