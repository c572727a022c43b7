"""Frames whose inputs arrive in host memory, pipelined (an extension of
Tina's API for rendering a stream of frames).

Each frame is an upload of its inputs from pinned host memory into a Scene's
device buffers (the in-place `set_face_*` copies), `Scene.render`, and the read
of `scene.img` back into pinned host memory.  On one stream these three run
back to back, and the GPU idles while the copy engines work.  FramePipeline
keeps `len(scenes)` Scene replicas, each with its own CUDA stream and pinned
host image, and gives frames to them in turn, so that frame k+1's upload runs
while frame k renders and frame k-1's image comes back.
"""
import torch

from ._device import require_cuda


class FramePipeline:
    """`FramePipeline(scenes)`: `scenes` are replicas of one scene (same
    resolution and objects, separate device buffers).  `submit(upload)` queues
    a frame on the next replica; `upload(scene)` issues that frame's input copies
    (for example `mesh.set_face_verts(pinned_host_array)` on the replica's
    mesh) and runs with the replica's stream current.  `result(k)` waits for
    frame k and returns its image in pinned host memory, valid until frame
    k + len(scenes) is submitted.  Host input arrays must stay unchanged until
    their frame's result has been collected."""

    def __init__(self, scenes):
        require_cuda('FramePipeline')
        if not scenes:
            raise ValueError('FramePipeline needs at least one scene')
        self.slots = []
        for scene in scenes:
            W, H = scene.res
            self.slots.append({
                'scene': scene,
                'stream': torch.cuda.Stream(),
                'img': torch.empty((W, H, 3), dtype=torch.float32).pin_memory(),
                'done': torch.cuda.Event(),
                'frame': -1,
            })
        self.submitted = 0

    def submit(self, upload):
        """Queues the next frame; returns its index."""
        k = self.submitted
        slot = self.slots[k % len(self.slots)]
        if slot['frame'] >= 0:
            # the replica's previous frame must be complete before its buffers
            # and host image are reused
            slot['done'].synchronize()
        with torch.cuda.stream(slot['stream']):
            upload(slot['scene'])
            slot['scene'].render()
            slot['img'].copy_(slot['scene'].img, non_blocking=True)
            slot['done'].record(slot['stream'])
        slot['frame'] = k
        self.submitted += 1
        return k

    def result(self, k):
        """Image of frame k (pinned host float32 [W, H, 3])."""
        slot = self.slots[k % len(self.slots)]
        if slot['frame'] != k:
            raise ValueError(f'frame {k} is not held (its replica now holds frame {slot["frame"]})')
        slot['done'].synchronize()
        return slot['img']

    def synchronize(self):
        for slot in self.slots:
            slot['stream'].synchronize()
