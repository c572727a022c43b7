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
        # the frame's packed (depth, face id) keys of the three-method raster
        # protocol (int64 [W, H], -1 = empty) and the next free face id
        self.keys = None
        self._face_cursor = 0

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
        """Engine.clear_depth (tina/core/engine.py:68-70): depth = maxdepth, and
        the frame's depth keys emptied; face ids restart at 0."""
        dev = default_device()
        if self.depth is None or tuple(self.depth.shape) != self.res:
            self.depth = torch.empty(self.res, dtype=torch.int32, device=dev)
        self.depth.fill_(self.maxdepth)
        if self.keys is None or tuple(self.keys.shape) != self.res:
            self.keys = torch.empty(self.res, dtype=torch.int64, device=dev)
        lib = N.load()
        N.check(lib.t3_clear(self.keys.data_ptr(), self.keys.numel(),
                             torch.cuda.current_stream().cuda_stream), 't3_clear')
        self._face_cursor = 0

    def _claim_faces(self, n):
        """First face id of the next object rasterised in this frame."""
        base = self._face_cursor
        if base + n >= 0xFFFFFFFF:
            raise ValueError('more than 2**32 - 1 faces in one frame')
        self._face_cursor = base + n
        return base

    def _keys_to_depth(self):
        """engine.depth from the packed keys: the high word holds the int32
        depth with its sign bit flipped, i.e. depth + 2**31; empty pixels keep
        maxdepth."""
        d = ((self.keys >> 32) & 0xFFFFFFFF) - (1 << 31)
        self.depth.copy_(torch.where(self.keys == -1, torch.full_like(d, self.maxdepth), d))

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
