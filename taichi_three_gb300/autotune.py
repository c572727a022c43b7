"""A small autotuner: time candidate launch configurations on the real
workload and keep the fastest.

Each candidate is a dict of keyword arguments.  `tune(key, candidates, run)`
calls run(candidate) once to warm up, then `repeats` times between CUDA events
on the current stream, and records the median.  Results are cached in memory
by `key` (a hashable signature of the workload) and, when the tuner has a path,
in a JSON file so later processes reuse them (opt-in: TINA3_AUTOTUNE_CACHE or
Autotuner(path=...)).

tune_scene() picks the raster mode of a Scene: direct, or binned with tile
8 / 16 / 32 and the automatic or doubled bin capacity.
"""
import json
import os

import torch


def cuda_event_timer(fn):
    """Milliseconds of fn() between CUDA events on the current stream."""
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


class Autotuner:
    def __init__(self, path=None, timer=None):
        self.path = path
        self.timer = timer or cuda_event_timer
        self.cache = {}
        if path and os.path.exists(path):
            with open(path) as f:
                for k, v in json.load(f).items():
                    self.cache[k] = (v['config'], v['ms'])

    @staticmethod
    def _key(key):
        return repr(key)

    def time(self, run, candidate, repeats=3):
        run(candidate)  # warm-up (also builds workspaces)
        times = [self.timer(lambda: run(candidate)) for _ in range(repeats)]
        times.sort()
        return times[len(times) // 2]

    def tune(self, key, candidates, run, repeats=3, force=False):
        """Returns (best candidate, its median ms); `self.log` keeps every timing."""
        k = self._key(key)
        if not force and k in self.cache:
            return self.cache[k]
        self.log = []
        best = None
        for c in candidates:
            ms = self.time(run, c, repeats)
            self.log.append((dict(c), ms))
            if best is None or ms < best[1]:
                best = (dict(c), ms)
        self.cache[k] = best
        if self.path:
            data = {kk: {'config': v[0], 'ms': v[1]} for kk, v in self.cache.items()}
            with open(self.path, 'w') as f:
                json.dump(data, f, indent=1)
        return best


_default = None


def default_tuner():
    global _default
    if _default is None:
        _default = Autotuner(os.environ.get('TINA3_AUTOTUNE_CACHE'))
    return _default


SCENE_CANDIDATES = ([dict(raster='direct')] +
                    [dict(raster='binned', tile=t, bin_scale=s) for t in (8, 16, 32) for s in (1, 2)])


def tune_scene(scene, candidates=None, tuner=None, repeats=3):
    """Chooses scene.raster_mode / tile / bin_capacity by timing scene.render()
    on the current scene.  Returns (config, ms)."""
    from . import _native as N
    import ctypes as C
    tuner = tuner or default_tuner()
    lib = N.load()
    nf = sum(obj.get_nfaces() if hasattr(obj, 'get_nfaces') else 0 for obj in scene.objects)
    key = ('scene', tuple(scene.res), int(nf), scene.tonemap)

    def apply(c):
        scene.raster_mode = c['raster']
        if c['raster'] == 'binned':
            scene.tile = c['tile']
            sc, _ = scene.describe()
            cap = C.c_int64()
            N.check(lib.t3_bin_capacity(C.byref(sc), scene.tile, 0, C.byref(cap)), 't3_bin_capacity')
            scene.bin_capacity = int(cap.value) * c.get('bin_scale', 1)

    def run(c):
        apply(c)
        scene.render()

    best, ms = tuner.tune(key, candidates or SCENE_CANDIDATES, run, repeats=repeats)
    apply(best)
    return best, ms
