"""Paint effects of a draw path: blend modes, gradients and image patterns.

Mirrors the reference's BlendMode (content/src/effects.rs:99-160), Gradient
and ColorStop (content/src/gradient.rs:27-72, 121-260), Pattern with an image
source and its filters (content/src/pattern.rs, effects.rs:64-95).  A draw
path's paint is its solid colour, or that colour as the base colour of a
gradient or pattern overlay (Paint, renderer/src/paint.rs:52-150: the
overlay's texel colour with its alpha times the base colour's alpha).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from enum import IntEnum

import numpy as np

from . import _abi

BlendMode = IntEnum("BlendMode", {name.upper(): i for i, name in enumerate(_abi.BLEND_MODES)})
BlendMode.__doc__ = "content/src/effects.rs:99-160 (SRC_OVER is 0 here)."


def blend_mode_is_destructive(mode: int) -> bool:
    """BlendMode::is_destructive (content/src/effects.rs:233-262)."""
    return BlendMode(mode) in (BlendMode.CLEAR, BlendMode.COPY, BlendMode.SRC_IN, BlendMode.DEST_IN,
                               BlendMode.SRC_OUT, BlendMode.DEST_ATOP)


def blend_mode_occludes_backdrop(mode: int) -> bool:
    """BlendMode::occludes_backdrop (content/src/effects.rs:202-230)."""
    return BlendMode(mode) in (BlendMode.SRC_OVER, BlendMode.CLEAR)


class GradientWrap(IntEnum):
    """content/src/gradient.rs:74-81."""
    CLAMP = _abi.PF_GRADIENT_WRAP_CLAMP
    REPEAT = _abi.PF_GRADIENT_WRAP_REPEAT


class GradientKind(IntEnum):
    LINEAR = _abi.PF_GRADIENT_LINEAR
    RADIAL = _abi.PF_GRADIENT_RADIAL


@dataclass(frozen=True)
class ColorStop:
    """content/src/gradient.rs:38-44."""
    color: object  # ColorU
    offset: float


def _f32(x) -> np.float32:
    return np.float32(x)


def _transform_point(t, x, y):
    """Transform2F * Vector2F in single precision (geometry/src/transform2d.rs:123-129, 312-318)."""
    x, y = _f32(x), _f32(y)
    return ((_f32(t[0]) * x + _f32(t[1]) * y) + _f32(t[4]),
            (_f32(t[2]) * x + _f32(t[3]) * y) + _f32(t[5]))


def _transform_mul(a, b):
    """Transform2F * Transform2F (geometry/src/transform2d.rs:115-121, 301-310); tuples are
    (m00, m01, m10, m11, tx, ty) in row-major naming."""
    a = [_f32(v) for v in a]
    b = [_f32(v) for v in b]
    m00 = a[0] * b[0] + a[1] * b[2]
    m10 = a[2] * b[0] + a[3] * b[2]
    m01 = a[0] * b[1] + a[1] * b[3]
    m11 = a[2] * b[1] + a[3] * b[3]
    tx, ty = _transform_point(a, b[4], b[5])
    return (m00, m01, m10, m11, tx, ty)


def _as_tuple(t):
    if t is None:
        return (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
    if hasattr(t, "m00"):
        return (t.m00, t.m01, t.m10, t.m11, t.tx, t.ty)
    return tuple(float(v) for v in t)


@dataclass(eq=False)
class Gradient:
    """A linear or radial gradient in scene coordinates (content/src/gradient.rs:27-72).

    Linear: the line ``from_`` -> ``to``.  Radial: the line between the two
    circles' centres, their radii, and ``transform`` (gradient space -> scene).
    """
    kind: GradientKind
    from_: tuple[float, float]
    to: tuple[float, float]
    radii: tuple[float, float] = (0.0, 0.0)
    transform: tuple = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
    wrap: GradientWrap = GradientWrap.CLAMP
    stops: list = field(default_factory=list)

    @classmethod
    def linear(cls, from_, to) -> "Gradient":
        """Gradient::linear / linear_from_points (content/src/gradient.rs:121-138)."""
        return cls(GradientKind.LINEAR, tuple(from_), tuple(to))

    linear_from_points = linear

    @classmethod
    def radial(cls, line, radii) -> "Gradient":
        """Gradient::radial (content/src/gradient.rs:140-156): ``line`` is a centre
        point, or a pair of centres."""
        line = tuple(line)
        if len(line) == 2 and not hasattr(line[0], "__len__"):
            a = b = line
        else:
            a, b = tuple(line[0]), tuple(line[1])
        return cls(GradientKind.RADIAL, tuple(a), tuple(b), (float(radii[0]), float(radii[1])))

    def add(self, stop: ColorStop) -> None:
        """Gradient::add (content/src/gradient.rs:158-164): after every stop with an
        offset <= the new one."""
        i = 0
        while i < len(self.stops) and self.stops[i].offset <= stop.offset:
            i += 1
        self.stops.insert(i, stop)

    def add_color_stop(self, color, offset: float) -> None:
        self.add(ColorStop(color, float(offset)))

    def set_wrap(self, wrap: GradientWrap) -> None:
        self.wrap = GradientWrap(wrap)

    def apply_transform(self, new_transform) -> None:
        """Gradient::apply_transform (content/src/gradient.rs:226-242)."""
        t = _as_tuple(new_transform)
        if t == (1.0, 0.0, 0.0, 1.0, 0.0, 0.0):
            return
        if self.kind == GradientKind.LINEAR:
            self.from_ = tuple(float(v) for v in _transform_point(t, *self.from_))
            self.to = tuple(float(v) for v in _transform_point(t, *self.to))
        else:
            self.transform = tuple(float(v) for v in _transform_mul(t, self.transform))

    def is_opaque(self) -> bool:
        """content/src/gradient.rs:215-217."""
        return all(s.color.a == 255 for s in self.stops)

    def to_c(self):
        """(PFCUDAGradient, the stops array it points at: keep both alive)."""
        stops = (_abi.PFCUDAColorStop * max(1, len(self.stops)))()
        for i, s in enumerate(self.stops):
            stops[i].offset = s.offset
            stops[i].color = _abi.PFColorU(s.color.r, s.color.g, s.color.b, s.color.a)
        g = _abi.PFCUDAGradient()
        g.kind, g.wrap = int(self.kind), int(self.wrap)
        g.from_ = _abi.PFVector2F(*self.from_)
        g.to = _abi.PFVector2F(*self.to)
        g.radius0, g.radius1 = self.radii
        t = self.transform
        g.transform = _abi.PFTransform2F(t[0], t[1], t[2], t[3], _abi.PFVector2F(t[4], t[5]))
        g.stops = C.addressof(stops) if self.stops else None
        g.stop_count = len(self.stops)
        return g, stops


class PatternFilterKind(IntEnum):
    """PatternFilter (content/src/effects.rs:64-95) without the text filter."""
    NONE = _abi.PF_PATTERN_FILTER_NONE
    BLUR_X = _abi.PF_PATTERN_FILTER_BLUR_X
    BLUR_Y = _abi.PF_PATTERN_FILTER_BLUR_Y
    COLOR_MATRIX = _abi.PF_PATTERN_FILTER_COLOR_MATRIX


@dataclass(eq=False)
class Pattern:
    """An image pattern (content/src/pattern.rs:21-200, PatternSource::Image).

    ``pixels``: (height, width, 4) uint8 straight-alpha RGBA; ``transform``:
    pattern space -> scene, (m00, m01, m10, m11, tx, ty)."""
    pixels: np.ndarray
    transform: tuple = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
    repeat_x: bool = False
    repeat_y: bool = False
    smoothing: bool = True
    filter: PatternFilterKind = PatternFilterKind.NONE
    blur_sigma: float = 0.0
    color_matrix: tuple = tuple([1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0, 1.0, 0, 0, 0, 0])

    @classmethod
    def from_image(cls, pixels) -> "Pattern":
        """Pattern::from_image (content/src/pattern.rs:97-99): identity transform, no filter."""
        return cls(np.ascontiguousarray(pixels, np.uint8))

    def apply_transform(self, transform) -> None:
        """Pattern::apply_transform (content/src/pattern.rs:119-122): after the existing one."""
        self.transform = tuple(float(v) for v in _transform_mul(_as_tuple(transform), self.transform))

    def set_blur(self, sigma: float, direction: str = "x") -> None:
        self.filter = PatternFilterKind.BLUR_X if direction == "x" else PatternFilterKind.BLUR_Y
        self.blur_sigma = float(sigma)

    def set_color_matrix(self, columns) -> None:
        """Five RGBA columns (the feColorMatrix layout: out = M * colour + column 4)."""
        m = np.asarray(columns, np.float32).reshape(20)
        self.filter = PatternFilterKind.COLOR_MATRIX
        self.color_matrix = tuple(float(v) for v in m)

    def is_opaque(self) -> bool:
        """Image::is_opaque (content/src/pattern.rs:208-212)."""
        return bool((np.asarray(self.pixels)[..., 3] == 255).all())

    def to_c(self):
        """(PFCUDAPattern, the pixel array it points at: keep both alive)."""
        px = np.ascontiguousarray(self.pixels, np.uint8)
        if px.ndim != 3 or px.shape[2] != 4:
            raise ValueError("pattern pixels must be (height, width, 4) uint8")
        p = _abi.PFCUDAPattern()
        p.pixels = px.ctypes.data
        p.height, p.width = px.shape[0], px.shape[1]
        t = self.transform
        p.transform = _abi.PFTransform2F(t[0], t[1], t[2], t[3], _abi.PFVector2F(t[4], t[5]))
        p.flags = ((_abi.PF_PATTERN_REPEAT_X if self.repeat_x else 0) | (_abi.PF_PATTERN_REPEAT_Y if self.repeat_y else 0)
                   | (0 if self.smoothing else _abi.PF_PATTERN_NO_SMOOTHING))
        p.filter = int(self.filter)
        p.blur_sigma = self.blur_sigma
        for k in range(20):
            p.color_matrix[k] = self.color_matrix[k]
        return p, px
