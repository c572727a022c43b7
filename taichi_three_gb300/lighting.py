"""Lamps and ambient light (tina/core/lighting.py:24-98)."""
import numpy as np

from . import _native as N


class Lighting:
    """Up to `maxlights` lamps: directional (dir, w = 0, normalised on the host in
    float64 like set_light, tina/core/lighting.py:55-65) or point (pos, w = 1),
    plus an ambient colour."""

    def __init__(self, maxlights=16):
        if maxlights > N.T3_MAX_LIGHTS:
            raise ValueError(f'at most {N.T3_MAX_LIGHTS} lights are supported')
        self.maxlights = maxlights
        self.light_dirs = np.tile(np.array([0, 0, 1, 0], dtype=np.float32), (maxlights, 1))
        self.light_colors = np.ones((maxlights, 3), dtype=np.float32)
        self.ambient_color = np.zeros(3, dtype=np.float32)
        self.nlights = 0

    def set_lights(self, light_dirs):
        if len(light_dirs) > self.maxlights:
            raise ValueError('too many lights')
        self.nlights = len(light_dirs)
        for i, (dir, color) in enumerate(light_dirs):
            self.light_dirs[i] = np.asarray(dir, dtype=np.float32)
            self.light_colors[i] = np.asarray(color, dtype=np.float32)

    def clear_lights(self):
        self.nlights = 0

    def add_light(self, dir=(0, 0, 1), pos=None, color=(1, 1, 1)):
        i = self.nlights
        if i >= self.maxlights:
            raise ValueError(f'at most {self.maxlights} lights')
        self.nlights = i + 1
        self.set_light(i, dir, pos, color)
        return i

    def set_light(self, i, dir=(0, 0, 1), pos=None, color=(1, 1, 1)):
        """Lamp i: a point lamp at `pos` (w = 1), or without `pos` a
        directional lamp along `dir`, normalised in float64 (w = 0); stored
        rounded to float32 like Taichi's field assignment."""
        if pos is None:
            v = np.asarray(dir, dtype=np.float64)
            xyzw = np.append(v / np.linalg.norm(v), 0.0)
        else:
            xyzw = np.append(np.asarray(pos, dtype=np.float64), 1.0)
        self.light_dirs[i] = xyzw.astype(np.float32)
        self.light_colors[i] = np.asarray(color, dtype=np.float64).astype(np.float32)

    def set_ambient_light(self, color):
        self.ambient_color = np.array(np.array(color, dtype=np.float64).tolist(),
                                      dtype=np.float32) * np.ones(3, dtype=np.float32)

    def _t3_fill(self, lt):
        lt.mode = N.T3_LIGHT_LAMPS
        lt.nlights = self.nlights
        for k in range(3):
            lt.ambient[k] = float(self.ambient_color[k])
        for i in range(self.nlights):
            for k in range(4):
                lt.lights[i].dir[k] = float(self.light_dirs[i, k])
            for k in range(3):
                lt.lights[i].color[k] = float(self.light_colors[i, k])
