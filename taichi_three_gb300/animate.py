"""Many frames in one CUDA graph.

FrameGraph captures `frames` consecutive frames of a Scene -- per frame the
device-side update (e.g. MeshGrid.displace_wave(t)), the mesh pre_compute
(grid normals), the frame's render and a per-frame checksum of scene.img --
into one CUDA graph, so replaying the animation costs one graph launch.
(Tina animates by calling scene.render() from a Python loop once per frame,
e.g. examples/meshgrid_cloth.py; no reference counterpart for the graph.)
"""
import torch


class FrameGraph:
    def __init__(self, scene, frames, update=None, checksums=True):
        self.scene = scene
        self.frames = int(frames)
        self.update = update
        self.checksums = checksums
        self.graph = None
        self.sums = None

    def _frame(self, k):
        if self.update is not None:
            self.update(k)
        self.scene.render()
        if self.checksums:
            self.sums[k] = self.scene.img.sum(dtype=torch.float64)

    def capture(self):
        """Warms up (allocates every workspace and output), then records the
        frames on a side stream."""
        dev = self.scene.engine.depth.device if self.scene.engine.depth is not None else 'cuda'
        self.sums = torch.zeros(self.frames, dtype=torch.float64, device='cuda')
        check = self.scene.check_bins
        self.scene.check_bins = False  # no host reads of the status inside the graph
        try:
            self._frame(0)
            torch.cuda.synchronize()
            stream = torch.cuda.Stream()
            stream.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(stream):
                self._frame(0)
                torch.cuda.synchronize()
                self.graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(self.graph, stream=stream):
                    for k in range(self.frames):
                        self._frame(k)
            torch.cuda.synchronize()
        finally:
            self.scene.check_bins = check
        del dev
        return self

    def replay(self):
        """Runs all captured frames (asynchronously on the current stream)."""
        if self.graph is None:
            self.capture()
        self.graph.replay()
