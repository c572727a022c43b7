"""Many views in one launch: BatchRenderer over t3_render_batch.

No reference counterpart (Tina renders one Scene per Scene.render call,
tina/scene/raster.py:168-207).  A BatchRenderer holds up to 64 Scenes (each
with its own resolution, camera, objects and lamps) and renders all of them
with two CUDA launches over all of them: direct, a persistent rasterisation
launch and a persistent shading launch whose CTAs take work items from global
queues; binned, one launch binning every scene's faces into its tiles and a
persistent launch rasterising and shading (scene, tile) items;
each Scene's img / face_id / depth / depth_f are written
exactly as Scene.render would write them.  BatchRenderer.autotune times the
direct work-item sizes and the binned tile size, threads per tile and bin
capacity on the actual batch and keeps the fastest.
"""
import ctypes as C

import torch

from . import _native as N
from ._device import default_device, require_cuda
from .autotune import default_tuner


def _stream():
    return torch.cuda.current_stream().cuda_stream


class BatchRenderer:
    """raster 'direct' (work items of faces_per_item faces and pixels_per_item
    pixels) or 'binned' (tiles of `tile` pixels, `tile_threads` threads per
    tile CTA, bin_capacity entries per tile bin: 0 for each scene's automatic
    size, -k for k times it); ctas_per_sm caps the resident CTAs of either."""

    def __init__(self, scenes, faces_per_item=1024, pixels_per_item=4096, ctas_per_sm=0, raster='direct',
                 tile=16, tile_threads=0, bin_capacity=0):
        self.scenes = list(scenes)
        if not 1 <= len(self.scenes) <= N.T3_BATCH_MAX_SCENES:
            raise ValueError(f'a batch holds 1..{N.T3_BATCH_MAX_SCENES} scenes')
        if raster not in ('direct', 'binned'):
            raise ValueError("raster must be 'direct' or 'binned'")
        self.config = dict(faces_per_item=faces_per_item, pixels_per_item=pixels_per_item,
                           ctas_per_sm=ctas_per_sm, raster=raster, tile=tile, tile_threads=tile_threads,
                           bin_capacity=bin_capacity)
        self._ws = None
        self._status = None
        self._keep = []

    @staticmethod
    def _t3_config(config):
        c = dict(config)
        c['raster'] = N.T3_RASTER_BINNED if c.get('raster', 'direct') == 'binned' else N.T3_RASTER_DIRECT
        return N.t3_batch_config(**c)

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

    def render(self, config=None, check_bins=True):
        """Renders every scene of the batch (two launches over all of them).  A
        binned batch whose bins overflowed is rendered again with bins twice
        the automatic size, then four times (check_bins=False skips the check,
        which reads the device status; inside a CUDA graph capture, for one)."""
        require_cuda('BatchRenderer.render')
        lib = N.load()
        dev = default_device()
        descs, outs, keep = self._describe(dev)
        n = len(self.scenes)
        config = dict(config or self.config)
        for attempt in range(3):
            cfg = self._t3_config(config)
            size = C.c_size_t()
            N.check(lib.t3_batch_workspace_size(descs, n, C.byref(cfg), C.byref(size)),
                    't3_batch_workspace_size')
            if self._ws is None or self._ws.numel() < size.value:
                self._ws = torch.empty(size.value, dtype=torch.uint8, device=dev)
            if self._status is None:
                self._status = torch.zeros(1, dtype=torch.int32, device=dev)
            N.check(lib.t3_render_batch(descs, outs, n, C.byref(cfg), self._ws.data_ptr(),
                                        self._ws.numel(), self._status.data_ptr(), _stream()),
                    't3_render_batch')
            if config.get('raster') != 'binned' or not check_bins:
                break
            if not (self.status() & N.T3_STATUS_BIN_OVERFLOW):
                break
            config['bin_capacity'] = -2 * (2 ** attempt)
        self._keep = keep
        self.last_config = config

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

    # the direct path's work-item sizes, and the binned path's tile size x
    # threads per tile x bin capacity (the automatic size, or twice it)
    CANDIDATES = ([dict(raster='direct', faces_per_item=f, pixels_per_item=p, ctas_per_sm=0)
                   for f in (256, 1024, 4096) for p in (1024, 4096, 16384)] +
                  [dict(raster='binned', tile=t, tile_threads=th, bin_capacity=b)
                   for t, th in ((8, 64), (16, 128), (16, 256), (32, 128), (32, 256)) for b in (0, -2)])

    def autotune(self, candidates=None, tuner=None, repeats=3):
        """Times each candidate configuration on this batch (CUDA events,
        median of `repeats` after one warm-up) and keeps the fastest; the
        result is cached by the batch signature.  A binned candidate whose
        bins overflow is not eligible.  Returns (config, ms)."""
        tuner = tuner or default_tuner()
        cands = [dict(c) for c in (candidates or self.CANDIDATES)]
        ok = []
        for c in cands:
            if c.get('raster') == 'binned':
                self.render(c, check_bins=False)
                if self.status() & N.T3_STATUS_BIN_OVERFLOW:
                    continue
            ok.append(c)
        best, ms = tuner.tune(self.signature(), ok, lambda c: self.render(c, check_bins=False),
                              repeats=repeats)
        self.config = dict(best)
        return self.config, ms
