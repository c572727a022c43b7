"""Many views in one launch: BatchRenderer over t3_render_batch.

No reference counterpart (Tina renders one Scene per Scene.render call,
tina/scene/raster.py:168-207).  A BatchRenderer holds up to 64 Scenes (each
with its own resolution, camera, objects and lamps) and renders all of them
with two persistent CUDA launches -- every scene's rasterisation in one, every
scene's shading in the next -- whose CTAs take work items from global queues;
each Scene's img / face_id / depth / depth_f are written
exactly as Scene.render would write them.  BatchRenderer.autotune times the
work-item sizes and residency on the actual batch and keeps the fastest.
"""
import ctypes as C

import torch

from . import _native as N
from ._device import default_device, require_cuda
from .autotune import default_tuner


def _stream():
    return torch.cuda.current_stream().cuda_stream


class BatchRenderer:
    def __init__(self, scenes, faces_per_item=1024, pixels_per_item=4096, ctas_per_sm=0):
        self.scenes = list(scenes)
        if not 1 <= len(self.scenes) <= N.T3_BATCH_MAX_SCENES:
            raise ValueError(f'a batch holds 1..{N.T3_BATCH_MAX_SCENES} scenes')
        self.config = dict(faces_per_item=faces_per_item, pixels_per_item=pixels_per_item,
                           ctas_per_sm=ctas_per_sm)
        self._ws = None
        self._status = None
        self._keep = []

    def _describe(self, dev):
        n = len(self.scenes)
        descs = (N.t3_scene * n)()
        outs = (N.t3_outputs * n)()
        keep = []
        for i, scene in enumerate(self.scenes):
            for obj in scene.objects:
                obj.pre_compute()
            sc, k = scene.describe(dev)
            keep.append(k)
            descs[i] = sc
            scene._alloc_outputs(dev)
            outs[i].rgb = scene.image.data_ptr()
            outs[i].face_id = scene.face_id.data_ptr()
            outs[i].depth = scene.engine.depth.data_ptr()
            outs[i].depth_f = scene.depth_f.data_ptr()
        return descs, outs, keep

    def render(self, config=None):
        """Renders every scene of the batch (one raster launch, one shading launch)."""
        require_cuda('BatchRenderer.render')
        lib = N.load()
        dev = default_device()
        descs, outs, keep = self._describe(dev)
        n = len(self.scenes)
        size = C.c_size_t()
        N.check(lib.t3_batch_workspace_size(descs, n, C.byref(size)), 't3_batch_workspace_size')
        if self._ws is None or self._ws.numel() < size.value:
            self._ws = torch.empty(size.value, dtype=torch.uint8, device=dev)
        if self._status is None:
            self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        cfg = N.t3_batch_config(**(config or self.config))
        N.check(lib.t3_render_batch(descs, outs, n, C.byref(cfg), self._ws.data_ptr(),
                                    self._ws.numel(), self._status.data_ptr(), _stream()),
                't3_render_batch')
        self._keep = keep

    def status(self):
        lib = N.load()
        out = C.c_int32()
        N.check(lib.t3_read_status(self._status.data_ptr(), C.byref(out), _stream()), 't3_read_status')
        return out.value

    def signature(self):
        """What the best configuration depends on: resolutions and face counts."""
        sig = []
        for s in self.scenes:
            nf = sum(obj.get_nfaces() if hasattr(obj, 'get_nfaces') else 0 for obj in s.objects)
            sig.append((tuple(s.res), int(nf)))
        return ('batch', tuple(sig))

    CANDIDATES = [dict(faces_per_item=f, pixels_per_item=p, ctas_per_sm=c)
                  for f in (256, 1024, 4096) for p in (1024, 4096, 16384) for c in (0, 2)]

    def autotune(self, candidates=None, tuner=None, repeats=3):
        """Times each candidate configuration on this batch (CUDA events,
        median of `repeats` after one warm-up) and keeps the fastest; the
        result is cached by the batch signature.  Returns (config, ms)."""
        tuner = tuner or default_tuner()
        cands = candidates or self.CANDIDATES
        best, ms = tuner.tune(self.signature(), cands, lambda c: self.render(c), repeats=repeats)
        self.config = dict(best)
        return self.config, ms
