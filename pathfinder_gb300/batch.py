"""Scene batches: many independent scenes uploaded together and rendered by
one set of launches (PFCUDASceneUploadBatch / PFCUDARenderBatch)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .scene import RectF, Scene


def target(pitch: int, clip: tuple[int, int, int, int], out_offset: int = 0, origin: tuple[int, int] = (0, 0)):
    """PFCUDASceneTarget: scene pixel (x, y) in `clip` -> out_offset + (y-oy)*pitch + (x-ox)."""
    t = _abi.PFCUDASceneTarget()
    t.out_offset = out_offset
    t.pitch = pitch
    t.origin_x, t.origin_y = origin
    t.clip = _abi.PFRectI(_abi.PFVector2I(clip[0], clip[1]), _abi.PFVector2I(clip[2], clip[3]))
    return t


class SceneBatch:
    """A list of scenes with their output targets."""

    def __init__(self, scenes: list[Scene], targets: list | None = None):
        self.scenes = list(scenes)
        self.targets = targets
        n = len(self.scenes)
        # the array holds copies of the descriptors: the descriptors themselves
        # stay alive with the batch, with the buffers they point into
        self._desc_objs = [s.desc() for s in self.scenes]
        self._descs = (_abi.PFCUDASceneDesc * n)(*self._desc_objs)
        self._targets = None
        if targets is not None:
            if len(targets) != n:
                raise ValueError("one target per scene")
            self._targets = (_abi.PFCUDASceneTarget * n)(*targets)
        self.key = tuple((s.id, s.epoch) for s in self.scenes)

    def __len__(self):
        return len(self.scenes)

    @classmethod
    def packed(cls, scenes: list[Scene]) -> "SceneBatch":
        """Each scene into its own width x height image, packed one after
        another in one buffer (element offsets in `offsets`)."""
        targets, off = [], 0
        offsets = []
        for s in scenes:
            targets.append(target(s.width, (0, 0, s.width, s.height), out_offset=off))
            offsets.append(off)
            off += s.width * s.height
        b = cls(scenes, targets)
        b.offsets = offsets
        b.total_pixels = off
        return b

    @classmethod
    def glyphs_of(cls, atlas: Scene) -> "SceneBatch":
        """One scene per glyph of an atlas scene: the glyph's path alone, view
        box = its cell, written into the cell of the shared atlas image."""
        if atlas.cells is None:
            raise ValueError("the scene has no glyph cells")
        starts = atlas.contour_starts.astype(np.int64)
        scenes, targets = [], []
        for g, path in enumerate(atlas.draw_paths):
            fc, n = int(path["first_contour"]), int(path["contour_count"])
            p0, p1 = int(starts[fc]), int(starts[fc + n])
            s = Scene()
            s.points = atlas.points[p0:p1]
            s.flags = atlas.flags[p0:p1]
            s.contour_starts = (starts[fc:fc + n + 1] - p0).astype(np.uint32)
            rec = np.array(path).reshape(1).copy()
            rec["first_contour"] = 0
            s.draw_paths = rec
            c = atlas.cells[g]
            s.view_box = RectF(float(c["x0"]), float(c["y0"]), float(c["x1"]), float(c["y1"]))
            s.width, s.height = atlas.width, atlas.height
            scenes.append(s)
            targets.append(target(atlas.width, (int(c["x0"]), int(c["y0"]), int(c["x1"]), int(c["y1"]))))
        b = cls(scenes, targets)
        b.width, b.height = atlas.width, atlas.height
        return b

    def upload_args(self):
        return (C.cast(self._descs, C.c_void_p), C.cast(self._targets, C.c_void_p) if self._targets else None,
                len(self.scenes))
