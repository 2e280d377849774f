"""Stroke to fill: StrokeStyle, LineCap, LineJoin (content/src/stroke.rs:45-86)
and the batch conversion of outlines to the filled outlines of their strokes
(OutlineStrokeToFill, :24-190), run on the GPU by PFCUDAStrokeToFill; dashes
before it (OutlineDash, content/src/dash.rs:18-152) by PFCUDADashOutlines and
PFCUDAStrokeToFillDashed."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from enum import IntEnum

import numpy as np

from . import _abi
from .scene import Contour, Outline


class LineCap(IntEnum):
    BUTT = _abi.PF_LINE_CAP_BUTT
    SQUARE = _abi.PF_LINE_CAP_SQUARE
    ROUND = _abi.PF_LINE_CAP_ROUND


class LineJoin(IntEnum):
    MITER = _abi.PF_LINE_JOIN_MITER
    BEVEL = _abi.PF_LINE_JOIN_BEVEL
    ROUND = _abi.PF_LINE_JOIN_ROUND


@dataclass
class StrokeStyle:
    """StrokeStyle::default(): width 1, butt caps, miter joins with limit 10."""
    line_width: float = 1.0
    line_cap: LineCap = LineCap.BUTT
    line_join: LineJoin = LineJoin.MITER
    miter_limit: float = 10.0


class StrokeBatch:
    """Outlines with their styles as one host-memory PFCUDAStrokeInput, and
    their dash patterns as a PFCUDADashInput.  An item is ``(outline, style)``
    or ``(outline, style, dashes, dash_offset)``: ``dashes`` the alternating
    on/off lengths, used as given (empty: not dashed), ``dash_offset`` the
    phase.  ``style`` may be None when the batch is only dashed."""

    def __init__(self, items):
        pts, flags, cstarts, closed, ostarts, styles = [], [], [0], [], [0], []
        dashes, dstarts, offsets = [], [0], []
        n = 0
        for item in items:
            outline, style = item[0], item[1]
            pattern = list(item[2]) if len(item) > 2 and item[2] is not None else []
            dashes += [float(x) for x in pattern]
            dstarts.append(len(dashes))
            offsets.append(float(item[3]) if len(item) > 3 else 0.0)
            for c in outline.contours:
                pts.append(np.asarray(c.points, np.float32).reshape(-1, 2))
                flags.append(np.asarray(c.flags, np.uint8))
                n += len(c.points)
                cstarts.append(n)
                closed.append(1 if c.closed else 0)
            ostarts.append(len(closed))
            styles.append(style)
        self.points = np.ascontiguousarray(np.concatenate(pts) if pts else np.zeros((0, 2), np.float32))
        self.flags = np.ascontiguousarray(np.concatenate(flags) if flags else np.zeros((0,), np.uint8))
        self.contour_starts = np.asarray(cstarts, np.uint32)
        self.contour_closed = np.asarray(closed, np.uint8) if closed else np.zeros((1,), np.uint8)
        self.outline_starts = np.asarray(ostarts, np.uint32)
        self.styles = (_abi.PFCUDAStrokeStyle * max(1, len(styles)))()
        for i, st in enumerate(styles):
            st = st or StrokeStyle()
            self.styles[i] = _abi.PFCUDAStrokeStyle(float(st.line_width), int(st.line_cap), int(st.line_join),
                                                    float(st.miter_limit))
        self.outline_count = len(styles)
        self.contour_count = len(closed)
        self.dashes = np.asarray(dashes if dashes else [0.0], np.float32)
        self.dash_starts = np.asarray(dstarts, np.uint32)
        self.dash_offsets = np.asarray(offsets if offsets else [0.0], np.float32)
        self.dashed = bool(dashes)

    def dash_desc(self) -> _abi.PFCUDADashInput:
        d = _abi.PFCUDADashInput()
        d.dashes = self.dashes.ctypes.data
        d.dash_starts = self.dash_starts.ctypes.data
        d.offsets = self.dash_offsets.ctypes.data
        return d

    def desc(self) -> _abi.PFCUDAStrokeInput:
        d = _abi.PFCUDAStrokeInput()
        d.points = self.points.ctypes.data
        d.point_flags = self.flags.ctypes.data
        d.contour_starts = self.contour_starts.ctypes.data
        d.contour_closed = self.contour_closed.ctypes.data
        d.outline_starts = self.outline_starts.ctypes.data
        d.styles = C.addressof(self.styles)
        d.point_count = len(self.points)
        d.contour_count = self.contour_count
        d.outline_count = self.outline_count
        d.memory = _abi.PF_MEMORY_HOST
        return d


def outlines_from_buffers(points, flags, contour_starts, outline_starts, contour_closed=None) -> list[Outline]:
    """Split flat stroke (or dash) output back into one Outline per input
    outline; contours are closed unless ``contour_closed`` says otherwise."""
    out = []
    for o in range(len(outline_starts) - 1):
        ol = Outline()
        for c in range(int(outline_starts[o]), int(outline_starts[o + 1])):
            a, b = int(contour_starts[c]), int(contour_starts[c + 1])
            ct = Contour()
            ct.points = [(float(x), float(y)) for x, y in points[a:b]]
            ct.flags = [int(f) for f in flags[a:b]]
            ct.closed = True if contour_closed is None else bool(contour_closed[c])
            ol.contours.append(ct)  # empty contours are kept: the counts stay aligned
        out.append(ol)
    return out
