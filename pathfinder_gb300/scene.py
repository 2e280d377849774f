"""Host-side scene model: the shape of the reference's Scene / DrawPath /
ClipPath / Outline / Contour API (renderer/src/scene.rs:39-472,
content/src/outline.rs:17-41, :531-557), stored as flat numpy buffers that the
C ABI consumes without conversion.
"""
from __future__ import annotations

import ctypes as C
import itertools
from dataclasses import dataclass, field
from enum import IntEnum

import numpy as np

from . import _abi

_NEXT_SCENE_ID = itertools.count()

CONTROL_POINT_0 = 0x01
CONTROL_POINT_1 = 0x02


class FillRule(IntEnum):
    """content/src/fill.rs: FillRule::{Winding, EvenOdd}."""
    WINDING = 0
    EVEN_ODD = 1


@dataclass(frozen=True)
class ColorU:
    r: int
    g: int
    b: int
    a: int = 255

    def is_opaque(self) -> bool:  # color/src/lib.rs:76-78
        return self.a == 255


@dataclass(frozen=True)
class ColorF:
    r: float
    g: float
    b: float
    a: float


@dataclass
class RectF:
    x0: float
    y0: float
    x1: float
    y1: float


class Contour:
    """A contour of on-curve points and control points (content/src/outline.rs:23-28)."""

    def __init__(self):
        self.points: list[tuple[float, float]] = []
        self.flags: list[int] = []
        self.closed = False  # Contour::closed: whether a stroke joins the ends

    def push_endpoint(self, x: float, y: float) -> "Contour":
        self.points.append((x, y)); self.flags.append(0)
        return self

    def push_quadratic(self, cx: float, cy: float, x: float, y: float) -> "Contour":
        self.points += [(cx, cy), (x, y)]; self.flags += [CONTROL_POINT_0, 0]
        return self

    def push_cubic(self, c0x, c0y, c1x, c1y, x, y) -> "Contour":
        self.points += [(c0x, c0y), (c1x, c1y), (x, y)]
        self.flags += [CONTROL_POINT_0, CONTROL_POINT_1, 0]
        return self

    def close(self) -> "Contour":
        """Contour::close.  Fills treat every contour as closed
        (Outline::close_all_contours); strokes join a closed contour's ends
        instead of capping them."""
        self.closed = True
        return self


class Outline:
    def __init__(self, contours: list[Contour] | None = None):
        self.contours = list(contours or [])

    def push_contour(self, contour: Contour) -> None:
        if contour.points:  # Outline::push_contour skips empty contours
            self.contours.append(contour)


@dataclass
class DrawPath:
    """renderer/src/scene.rs:441-456, 509-583.  ``paint`` is the solid colour, or
    the base colour of ``gradient`` (only its alpha counts then: the gradient
    combines SrcIn over it); ``blend_mode`` is a BlendMode."""
    outline: Outline
    paint: ColorU = ColorU(0, 0, 0, 255)
    fill_rule: FillRule = FillRule.WINDING
    clip_path: int | None = None
    blend_mode: int = 0
    gradient: object = None  # paint.Gradient
    pattern: object = None   # paint.Pattern (a path takes a gradient or a pattern)


@dataclass
class ClipPath:
    """renderer/src/scene.rs:458-474, 585-612: a clip path may itself be
    clipped by a previously pushed clip path (a clip chain)."""
    outline: Outline
    fill_rule: FillRule = FillRule.WINDING
    clip_path: int | None = None


_FILL, _TILE, _CLIP, _PATH, _RECT = _abi.record_dtypes()


class Scene:
    """The vector scene (renderer/src/scene.rs:39-48) as flat buffers.

    ``points`` (N, 2) float32, ``flags`` (N,) uint8, ``contour_starts``
    (C + 1,) uint32, ``clip_paths`` / ``draw_paths`` structured arrays with the
    layout of PFCUDAPath, and the view box.  ``id``/``epoch`` drive the
    renderer's scene-upload cache (renderer/src/builder.rs:190-216).
    """

    def __init__(self):
        self.id = next(_NEXT_SCENE_ID)
        self.epoch = 0
        self.points = np.zeros((0, 2), np.float32)
        self.flags = np.zeros((0,), np.uint8)
        self.contour_starts = np.zeros((1,), np.uint32)
        self.clip_paths = np.zeros((0,), _PATH)
        self.draw_paths = np.zeros((0,), _PATH)
        self.view_box = RectF(0.0, 0.0, 0.0, 0.0)
        self.width = 0
        self.height = 0
        self.cells = None  # glyph atlas cells, when generated
        self.gradients: list = []  # paint.Gradient: overlays 1..len(gradients)
        self.patterns: list = []   # paint.Pattern: the overlays after the gradients
        self._pending: list = []

    # --- the reference's mutators -----------------------------------------
    def set_view_box(self, rect: RectF) -> None:
        self.view_box = rect
        self.width = int(np.ceil(rect.x1))
        self.height = int(np.ceil(rect.y1))
        self.epoch += 1

    def _append_outline(self, outline: Outline) -> tuple[int, int]:
        first = len(self.contour_starts) - 1
        pts, fl, starts = [self.points], [self.flags], [self.contour_starts]
        n = len(self.points)
        new_starts = []
        for c in outline.contours:
            pts.append(np.asarray(c.points, np.float32).reshape(-1, 2))
            fl.append(np.asarray(c.flags, np.uint8))
            n += len(c.points)
            new_starts.append(n)
        self.points = np.concatenate(pts)
        self.flags = np.concatenate(fl)
        self.contour_starts = np.concatenate([self.contour_starts, np.asarray(new_starts, np.uint32)])
        return first, len(outline.contours)

    def push_clip_path(self, clip: ClipPath) -> int:
        first, count = self._append_outline(clip.outline)
        rec = np.zeros((1,), _PATH)
        rec["first_contour"], rec["contour_count"] = first, count
        rec["clip_path"] = -1 if clip.clip_path is None else clip.clip_path
        rec["fill_rule"] = int(clip.fill_rule)
        self.clip_paths = np.concatenate([self.clip_paths, rec])
        self.epoch += 1
        return len(self.clip_paths) - 1

    def push_draw_path(self, path: DrawPath) -> int:
        first, count = self._append_outline(path.outline)
        rec = np.zeros((1,), _PATH)
        rec["first_contour"], rec["contour_count"] = first, count
        rec["paint"] = (path.paint.r, path.paint.g, path.paint.b, path.paint.a)
        rec["clip_path"] = -1 if path.clip_path is None else path.clip_path
        rec["fill_rule"] = int(path.fill_rule)
        rec["blend_mode"] = int(path.blend_mode)
        if path.gradient is not None and path.pattern is not None:
            raise ValueError("a draw path takes a gradient or a pattern, not both")
        if path.gradient is not None:
            rec["overlay"] = self.push_gradient(path.gradient) + 1
        elif path.pattern is not None:
            rec["overlay"] = self.PATTERN_OVERLAY_BASE + self.push_pattern(path.pattern)
        self.draw_paths = np.concatenate([self.draw_paths, rec])
        self.epoch += 1
        return len(self.draw_paths) - 1

    def push_gradient(self, gradient) -> int:
        """Index of ``gradient`` among the scene's gradients (added once per object,
        as Palette::push_paint dedupes paints, renderer/src/paint.rs:381-390)."""
        for i, g in enumerate(self.gradients):
            if g is gradient:
                return i
        if len(self.gradients) >= 0xfffe:
            raise ValueError("too many gradients in one scene")
        self.gradients.append(gradient)
        self.epoch += 1
        return len(self.gradients) - 1

    # Pattern overlays are recorded as BASE + index and numbered after the
    # gradients when the descriptor is made (the gradient count may still grow).
    PATTERN_OVERLAY_BASE = 0x8000

    def push_pattern(self, pattern) -> int:
        for i, p in enumerate(self.patterns):
            if p is pattern:
                return i
        if len(self.patterns) >= 0x7ffe:
            raise ValueError("too many patterns in one scene")
        self.patterns.append(pattern)
        self.epoch += 1
        return len(self.patterns) - 1

    # --- C ABI view -----------------------------------------------------------
    def desc(self) -> _abi.PFCUDASceneDesc:
        """PFCUDASceneDesc pointing at this scene's host buffers.  The same
        epoch and buffers give the same descriptor, built once."""
        for name in ("points", "flags", "contour_starts", "clip_paths", "draw_paths"):
            a = getattr(self, name)
            if not a.flags["C_CONTIGUOUS"]:
                setattr(self, name, np.ascontiguousarray(a))
        vb = self.view_box
        key = (self.epoch, vb.x0, vb.y0, vb.x1, vb.y1) + tuple(
            (a.ctypes.data, a.shape[0]) for a in (self.points, self.flags, self.contour_starts, self.clip_paths,
                                                  self.draw_paths))
        cached = getattr(self, "_desc_cache", None)
        if cached is not None and cached[0] == key:
            return cached[1]
        d = self._build_desc()
        # gradients and patterns are converted when the descriptor is made:
        # a scene with any is described afresh every time, so that edits of
        # those objects are seen
        self._desc_cache = (key, d) if not (self.gradients or self.patterns) else None
        return d

    def _build_desc(self) -> _abi.PFCUDASceneDesc:
        d = _abi.PFCUDASceneDesc()
        d.points = self.points.ctypes.data
        d.point_flags = self.flags.ctypes.data
        d.contour_starts = self.contour_starts.ctypes.data
        d.clip_paths = self.clip_paths.ctypes.data if len(self.clip_paths) else None
        d.draw_paths = self.draw_paths.ctypes.data if len(self.draw_paths) else None
        d.point_count = len(self.points)
        d.contour_count = len(self.contour_starts) - 1
        d.clip_path_count = len(self.clip_paths)
        d.draw_path_count = len(self.draw_paths)
        vb = self.view_box
        d.view_box = _abi.PFRectF(_abi.PFVector2F(vb.x0, vb.y0), _abi.PFVector2F(vb.x1, vb.y1))
        d.memory = _abi.PF_MEMORY_HOST
        keep = []
        if self.gradients:
            arr = (_abi.PFCUDAGradient * len(self.gradients))()
            keep.append(arr)
            for i, g in enumerate(self.gradients):
                arr[i], stops = g.to_c()
                keep.append(stops)
            d.gradients = C.addressof(arr)
            d.gradient_count = len(self.gradients)
        if self.patterns:
            parr = (_abi.PFCUDAPattern * len(self.patterns))()
            keep.append(parr)
            for i, p in enumerate(self.patterns):
                parr[i], px = p.to_c()
                keep.append(px)
            d.patterns = C.addressof(parr)
            d.pattern_count = len(self.patterns)
        ov = self.draw_paths["overlay"] if len(self.draw_paths) else np.zeros((0,), np.uint16)
        pat = ov >= self.PATTERN_OVERLAY_BASE
        if pat.any():  # the descriptor numbers the patterns after the gradients
            dp = self.draw_paths.copy()
            dp["overlay"][pat] = ov[pat] - self.PATTERN_OVERLAY_BASE + len(self.gradients) + 1
            keep.append(dp)
            d.draw_paths = dp.ctypes.data
        # the descriptor points into these: it holds them itself, so a
        # descriptor still in use (a frame in flight) outlives a newer one
        d._keep = keep
        return d

    @property
    def segment_count(self) -> int:
        """Input segments as ContourIter yields them (closing lines included)."""
        f = self.flags
        n = 0
        for c in range(len(self.contour_starts) - 1):
            a, b = int(self.contour_starts[c]), int(self.contour_starts[c + 1])
            if b > a:
                n += 1 + int(np.count_nonzero((f[a + 1:b] & 3) == 0))
        return n


def generate_scene(workload: int, seed: int = 1, scale: float = 1.0, jitter_sigma: float = 0.0,
                   jitter_seed: int = 0, width: int = 0, height: int = 0, lib=None) -> Scene:
    """A seeded synthetic scene (include/pathfinder_cuda_scenes.h).  `lib`: a
    loaded library exporting the generator (default: libpfscenes.so)."""
    L = lib if lib is not None else _abi.scenes_lib()

    def check(code, what):
        if code != _abi.PF_CUDA_OK:
            raise RuntimeError(f"{what} failed with status {code}")

    p = _abi.PFCUDASceneParams(workload, seed, scale, jitter_sigma, jitter_seed, width, height)
    h = C.c_void_p()
    check(L.PFCUDASceneGenerate(C.byref(p), C.byref(h)), "PFCUDASceneGenerate")
    try:
        d = _abi.PFCUDASceneDesc()
        w, hh = C.c_int32(), C.c_int32()
        check(L.PFCUDASceneGetDesc(h, C.byref(d), C.byref(w), C.byref(hh)), "PFCUDASceneGetDesc")
        s = Scene()
        npt, nc = d.point_count, d.contour_count

        def arr(ptr, ctype, count, dtype):
            if count == 0:
                return np.zeros((0,), dtype)
            buf = (ctype * count).from_address(ptr)
            return np.frombuffer(buf, dtype=dtype, count=count).copy()

        s.points = arr(d.points, C.c_float, 2 * npt, np.float32).reshape(-1, 2)
        s.flags = arr(d.point_flags, C.c_uint8, npt, np.uint8)
        s.contour_starts = arr(d.contour_starts, C.c_uint32, nc + 1, np.uint32)
        s.clip_paths = arr(d.clip_paths, C.c_uint8, d.clip_path_count * _PATH.itemsize, np.uint8).view(_PATH) \
            if d.clip_path_count else np.zeros((0,), _PATH)
        s.draw_paths = arr(d.draw_paths, C.c_uint8, d.draw_path_count * _PATH.itemsize, np.uint8).view(_PATH) \
            if d.draw_path_count else np.zeros((0,), _PATH)
        s.view_box = RectF(d.view_box.origin.x, d.view_box.origin.y, d.view_box.lower_right.x,
                           d.view_box.lower_right.y)
        s.width, s.height = w.value, hh.value
        if workload == _abi.PF_SCENE_GLYPH_ATLAS:
            n = d.draw_path_count
            cells = np.zeros((n,), _RECT)
            L.PFCUDASceneGetCells(h, cells.ctypes.data, n)
            s.cells = cells
        return s
    finally:
        L.PFCUDASceneDestroy(h)
