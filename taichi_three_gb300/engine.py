"""Engine: resolution, camera matrices, pixel bias, depth (tina/core/engine.py)."""
import numpy as np
import torch

from . import _native as N
from ._device import default_device


class Engine:
    def __init__(self, res_x=512, res_y=None):
        if res_y is None:
            res_y = res_x
        if isinstance(res_x, (tuple, list)):
            res_x, res_y = res_x
        self.res = (int(res_x), int(res_y))
        self.maxdepth = N.T3_MAXDEPTH
        # init_engine (tina/core/engine.py:20-26): W2V = V2W = diag(1, 1, -1, 1)
        self.W2V = np.diag(np.array([1, 1, -1, 1], dtype=np.float32))
        self.V2W = np.diag(np.array([1, 1, -1, 1], dtype=np.float32))
        self.bias = np.array([0.5, 0.5], dtype=np.float32)
        self.depth = None  # torch int32 [W, H] after a render

    def set_camera(self, view, proj):
        """W2V = proj @ view in float64, V2W its inverse, both stored as float32
        (tina/core/engine.py:72-76)."""
        W2V = np.asarray(proj, dtype=np.float64) @ np.asarray(view, dtype=np.float64)
        V2W = np.linalg.inv(W2V)
        self.W2V = np.array(W2V, dtype=np.float32)
        self.V2W = np.array(V2W, dtype=np.float32)

    def randomize_bias(self, center):
        if center:
            self.bias = np.array([0.5, 0.5], dtype=np.float32)
        else:
            self.bias = np.random.random(2).astype(np.float32)

    def clear_depth(self):
        if self.depth is None:
            self.depth = torch.empty(self.res, dtype=torch.int32, device=default_device())
        self.depth.fill_(self.maxdepth)

    def _t3_fill_frame(self, fr, flags, bgcolor):
        fr.width, fr.height = self.res
        fr.flags = flags
        fr.maxdepth = self.maxdepth
        w2v = self.W2V.reshape(-1)
        v2w = self.V2W.reshape(-1)
        for k in range(16):
            fr.W2V[k] = float(w2v[k])
            fr.V2W[k] = float(v2w[k])
        fr.bias[0], fr.bias[1] = float(self.bias[0]), float(self.bias[1])
        bg = np.broadcast_to(np.asarray(bgcolor, dtype=np.float32), (3,))
        for k in range(3):
            fr.bgcolor[k] = float(bg[k])
