"""A minimal SVG front-end: the role of the reference's svg crate
(svg/src/lib.rs:94-286, which walks a usvg tree) for documents made of paths
and basic shapes.

Supported: <svg> (width/height/viewBox), <g>, <path> (every path-data
command; quadratics, smooth curves and arcs become cubics as usvg makes them),
<rect> (with rx/ry), <circle>, <ellipse>, <line>, <polyline>, <polygon>,
<defs>, <linearGradient>/<radialGradient> with <stop>s (spreadMethod pad,
repeat, reflect as svg/src/lib.rs:233-261 builds them), one <clipPath> per
group (clip-path="url(#id)"), and the presentation attributes fill, stroke,
fill-opacity, stroke-opacity, fill-rule, stroke-width, stroke-linecap,
stroke-linejoin, stroke-miterlimit, stroke-dasharray, stroke-dashoffset,
transform, in attributes or in style="".
Fills become draw paths with the outline transformed; strokes are dashed
(OutlineDash, :159-164) and stroked in their local coordinates on the GPU
(PFCUDAStrokeToFill or PFCUDAStrokeToFillDashed, all strokes of the document
in one batch) and then transformed, as push_draw_path does (:264-286).
Stroke widths below 0.0333 use 0.0333 (HAIRLINE_STROKE_WIDTH, :38).
Unsupported elements (filters, masks, images, patterns, text, CSS classes) are
reported in `unsupported`.
"""
from __future__ import annotations

import math
import re
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

from .paint import BlendMode, Gradient, GradientWrap, ColorStop
from .scene import ClipPath, ColorU, Contour, DrawPath, FillRule, Outline, RectF, Scene
from .stroke import LineCap, LineJoin, StrokeStyle

HAIRLINE_STROKE_WIDTH = 0.0333

_NAMED = {
    "black": (0, 0, 0), "white": (255, 255, 255), "red": (255, 0, 0), "green": (0, 128, 0),
    "blue": (0, 0, 255), "yellow": (255, 255, 0), "cyan": (0, 255, 255), "magenta": (255, 0, 255),
    "gray": (128, 128, 128), "grey": (128, 128, 128), "orange": (255, 165, 0), "purple": (128, 0, 128),
    "brown": (165, 42, 42), "pink": (255, 192, 203), "lime": (0, 255, 0), "navy": (0, 0, 128),
    "teal": (0, 128, 128), "silver": (192, 192, 192), "maroon": (128, 0, 0), "olive": (128, 128, 0),
}

_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _tag(el) -> str:
    return el.tag.rsplit("}", 1)[-1]


# --- transforms: (a, b, c, d, e, f), x' = a x + c y + e, y' = b x + d y + f ------
def _mul(m, n):
    a, b, c, d, e, f = m
    A, B, C, D, E, F = n
    return (a * A + c * B, b * A + d * B, a * C + c * D, b * C + d * D, a * E + c * F + e, b * E + d * F + f)


IDENTITY = (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)


def parse_transform(text: str | None):
    m = IDENTITY
    if not text:
        return m
    for name, args in re.findall(r"(\w+)\s*\(([^)]*)\)", text):
        v = [float(x) for x in re.findall(_NUM, args)]
        if name == "matrix" and len(v) == 6:
            t = tuple(v)
        elif name == "translate":
            t = (1, 0, 0, 1, v[0], v[1] if len(v) > 1 else 0.0)
        elif name == "scale":
            t = (v[0], 0, 0, v[1] if len(v) > 1 else v[0], 0, 0)
        elif name == "rotate":
            r = math.radians(v[0])
            t = (math.cos(r), math.sin(r), -math.sin(r), math.cos(r), 0, 0)
            if len(v) == 3:
                t = _mul(_mul((1, 0, 0, 1, v[1], v[2]), t), (1, 0, 0, 1, -v[1], -v[2]))
        elif name == "skewX":
            t = (1, 0, math.tan(math.radians(v[0])), 1, 0, 0)
        elif name == "skewY":
            t = (1, math.tan(math.radians(v[0])), 0, 1, 0, 0)
        else:
            continue
        m = _mul(m, tuple(float(x) for x in t))
    return m


def _apply(m, x, y):
    return (m[0] * x + m[2] * y + m[4], m[1] * x + m[3] * y + m[5])


# --- colours ----------------------------------------------------------------------
def parse_color(text: str | None):
    """(r, g, b) or None for none/invalid; url(#id) handled by the caller."""
    if text is None:
        return None
    t = text.strip().lower()
    if t in ("none", "transparent", ""):
        return None
    if t.startswith("#"):
        h = t[1:]
        if len(h) == 3:
            return tuple(int(ch * 2, 16) for ch in h)
        if len(h) == 6:
            return tuple(int(h[i:i + 2], 16) for i in (0, 2, 4))
        return None
    mm = re.match(r"rgb\(\s*([^)]*)\)", t)
    if mm:
        parts = [p.strip() for p in mm.group(1).split(",")]
        out = []
        for p in parts[:3]:
            out.append(round(float(p[:-1]) * 2.55) if p.endswith("%") else int(float(p)))
        return tuple(max(0, min(255, v)) for v in out)
    return _NAMED.get(t)


# --- path data ----------------------------------------------------------------------
def _arc_to_cubics(x0, y0, rx, ry, phi_deg, large, sweep, x, y):
    """SVG elliptical arc (SVG 1.1 F.6.5-F.6.6) as cubics of at most 90 degrees."""
    if (x0, y0) == (x, y):
        return []
    rx, ry = abs(rx), abs(ry)
    if rx == 0 or ry == 0:
        return [("L", x, y)]
    phi = math.radians(phi_deg)
    cp, sp = math.cos(phi), math.sin(phi)
    dx, dy = (x0 - x) / 2, (y0 - y) / 2
    x1p, y1p = cp * dx + sp * dy, -sp * dx + cp * dy
    lam = (x1p / rx) ** 2 + (y1p / ry) ** 2
    if lam > 1:
        s = math.sqrt(lam)
        rx, ry = rx * s, ry * s
    num = rx * rx * ry * ry - rx * rx * y1p * y1p - ry * ry * x1p * x1p
    den = rx * rx * y1p * y1p + ry * ry * x1p * x1p
    co = math.sqrt(max(0.0, num / den)) if den else 0.0
    if large == sweep:
        co = -co
    cxp, cyp = co * rx * y1p / ry, -co * ry * x1p / rx
    cx, cy = cp * cxp - sp * cyp + (x0 + x) / 2, sp * cxp + cp * cyp + (y0 + y) / 2

    def ang(ux, uy, vx, vy):
        return math.atan2(ux * vy - uy * vx, ux * vx + uy * vy)

    t1 = ang(1, 0, (x1p - cxp) / rx, (y1p - cyp) / ry)
    dt = ang((x1p - cxp) / rx, (y1p - cyp) / ry, (-x1p - cxp) / rx, (-y1p - cyp) / ry)
    if not sweep and dt > 0:
        dt -= 2 * math.pi
    elif sweep and dt < 0:
        dt += 2 * math.pi
    n = max(1, int(math.ceil(abs(dt) / (math.pi / 2) - 1e-9)))
    h = dt / n
    k = 4.0 / 3.0 * math.tan(h / 4)
    out = []

    def pt(t):
        ex, ey = rx * math.cos(t), ry * math.sin(t)
        return cp * ex - sp * ey + cx, sp * ex + cp * ey + cy

    def dpt(t):
        ex, ey = -rx * math.sin(t), ry * math.cos(t)
        return cp * ex - sp * ey, sp * ex + cp * ey

    for i in range(n):
        a0, a1 = t1 + i * h, t1 + (i + 1) * h
        p0, p1 = pt(a0), pt(a1)
        d0, d1 = dpt(a0), dpt(a1)
        c0 = (p0[0] + k * d0[0], p0[1] + k * d0[1])
        c1 = (p1[0] - k * d1[0], p1[1] - k * d1[1])
        end = (x, y) if i == n - 1 else p1
        out.append(("C", c0[0], c0[1], c1[0], c1[1], end[0], end[1]))
    return out


def parse_path_data(d: str):
    """Path data -> list of contours: (points [(x, y, flags)], closed), absolute,
    with quadratics, smooth curves and arcs as cubics."""
    toks = re.findall(r"[MmLlHhVvCcSsQqTtAaZz]|" + _NUM, d or "")
    contours = []
    cur = None
    x = y = sx = sy = 0.0
    last_c2 = last_q = None
    i, cmd = 0, None

    def nums(k):
        nonlocal i
        v = [float(t) for t in toks[i:i + k]]
        i += k
        return v

    def start(px, py):
        nonlocal cur
        cur = ([(px, py, 0)], False)
        contours.append(cur)

    def ensure():
        if cur is None:
            start(x, y)

    while i < len(toks):
        t = toks[i]
        if re.match(r"[A-Za-z]", t):
            cmd = t
            i += 1
            if cmd in "Zz":
                if cur is not None:
                    contours[-1] = (cur[0], True)
                    cur = None
                x, y = sx, sy
                last_c2 = last_q = None
                continue
        elif cmd is None:
            break
        rel = cmd.islower()
        C = cmd.upper()
        ox, oy = (x, y) if rel else (0.0, 0.0)
        try:
            if C == "M":
                px, py = nums(2)
                x, y = px + ox, py + oy
                sx, sy = x, y
                start(x, y)
                cmd = "l" if rel else "L"  # following pairs are lines
                last_c2 = last_q = None
            elif C == "L":
                px, py = nums(2)
                x, y = px + ox, py + oy
                ensure(); cur[0].append((x, y, 0))
                last_c2 = last_q = None
            elif C == "H":
                (px,) = nums(1)
                x = px + ox
                ensure(); cur[0].append((x, y, 0))
                last_c2 = last_q = None
            elif C == "V":
                (py,) = nums(1)
                y = py + oy
                ensure(); cur[0].append((x, y, 0))
                last_c2 = last_q = None
            elif C in "CS":
                if C == "C":
                    x1, y1, x2, y2, px, py = nums(6)
                    c1 = (x1 + ox, y1 + oy)
                else:
                    x2, y2, px, py = nums(4)
                    c1 = (2 * x - last_c2[0], 2 * y - last_c2[1]) if last_c2 else (x, y)
                c2 = (x2 + ox, y2 + oy)
                ensure()
                cur[0].extend([(c1[0], c1[1], 1), (c2[0], c2[1], 2), (px + ox, py + oy, 0)])
                x, y = px + ox, py + oy
                last_c2, last_q = c2, None
            elif C in "QT":
                if C == "Q":
                    qx, qy, px, py = nums(4)
                    q = (qx + ox, qy + oy)
                else:
                    px, py = nums(2)
                    q = (2 * x - last_q[0], 2 * y - last_q[1]) if last_q else (x, y)
                ex, ey = px + ox, py + oy
                # quadratic -> cubic, as usvg converts it
                c1 = (x + 2.0 / 3.0 * (q[0] - x), y + 2.0 / 3.0 * (q[1] - y))
                c2 = (ex + 2.0 / 3.0 * (q[0] - ex), ey + 2.0 / 3.0 * (q[1] - ey))
                ensure()
                cur[0].extend([(c1[0], c1[1], 1), (c2[0], c2[1], 2), (ex, ey, 0)])
                x, y = ex, ey
                last_q, last_c2 = q, None
            elif C == "A":
                rx, ry, phi, large, sweep, px, py = nums(7)
                ex, ey = px + ox, py + oy
                ensure()
                for seg in _arc_to_cubics(x, y, rx, ry, phi, bool(large), bool(sweep), ex, ey):
                    if seg[0] == "L":
                        cur[0].append((seg[1], seg[2], 0))
                    else:
                        cur[0].extend([(seg[1], seg[2], 1), (seg[3], seg[4], 2), (seg[5], seg[6], 0)])
                x, y = ex, ey
                last_c2 = last_q = None
            else:
                i += 1
        except (ValueError, IndexError):
            break
    return [c for c in contours if c[0]]


# --- document walk ------------------------------------------------------------------
def _length(v, default=0.0):
    if v is None:
        return default
    m = re.match(_NUM, v.strip())
    return float(m.group(0)) if m else default


def _dasharray(v):
    """stroke-dasharray as usvg hands it to the reference (svg/src/lib.rs:159):
    "none", a negative length or a zero sum leave the stroke undashed, and an
    odd number of lengths is repeated once to make it even (SVG 1.1, 11.4)."""
    if v is None or v.strip() in ("", "none"):
        return None
    vals = [float(x) for x in re.findall(_NUM, v)]
    if not vals or any(x < 0 for x in vals) or sum(vals) <= 0:
        return None
    return vals * 2 if len(vals) % 2 else vals


def _style(el):
    """Presentation attributes of an element, style="" winning over attributes."""
    a = dict(el.attrib)
    for decl in (a.pop("style", "") or "").split(";"):
        if ":" in decl:
            k, v = decl.split(":", 1)
            a[k.strip()] = v.strip()
    return a


_INHERITED = ("fill", "stroke", "fill-opacity", "stroke-opacity", "fill-rule", "stroke-width", "stroke-linecap",
              "stroke-linejoin", "stroke-miterlimit", "stroke-dasharray", "stroke-dashoffset")


@dataclass
class _State:
    transform: tuple = IDENTITY
    clip: int | None = None
    attrs: dict = field(default_factory=lambda: {"fill": "black"})


def _shape_path(tag, a):
    """Basic shapes as path data (SVG 1.1 9.2-9.7)."""
    f = lambda k: _length(a.get(k))
    if tag == "rect":
        x, y, w, h = f("x"), f("y"), f("width"), f("height")
        if w <= 0 or h <= 0:
            return ""
        rx, ry = a.get("rx"), a.get("ry")
        rx = _length(rx) if rx is not None else (_length(ry) if ry is not None else 0.0)
        ry = _length(ry) if ry is not None else rx
        rx, ry = min(rx, w / 2), min(ry, h / 2)
        if rx <= 0 or ry <= 0:
            return f"M{x} {y}H{x + w}V{y + h}H{x}Z"
        return (f"M{x + rx} {y}H{x + w - rx}A{rx} {ry} 0 0 1 {x + w} {y + ry}V{y + h - ry}"
                f"A{rx} {ry} 0 0 1 {x + w - rx} {y + h}H{x + rx}A{rx} {ry} 0 0 1 {x} {y + h - ry}"
                f"V{y + ry}A{rx} {ry} 0 0 1 {x + rx} {y}Z")
    if tag in ("circle", "ellipse"):
        cx, cy = f("cx"), f("cy")
        rx = f("r") if tag == "circle" else f("rx")
        ry = f("r") if tag == "circle" else f("ry")
        if rx <= 0 or ry <= 0:
            return ""
        return (f"M{cx + rx} {cy}A{rx} {ry} 0 0 1 {cx} {cy + ry}A{rx} {ry} 0 0 1 {cx - rx} {cy}"
                f"A{rx} {ry} 0 0 1 {cx} {cy - ry}A{rx} {ry} 0 0 1 {cx + rx} {cy}Z")
    if tag == "line":
        return f"M{f('x1')} {f('y1')}L{f('x2')} {f('y2')}"
    if tag in ("polyline", "polygon"):
        v = [float(t) for t in re.findall(_NUM, a.get("points", ""))]
        if len(v) < 4:
            return ""
        d = "M" + " L".join(f"{v[i]} {v[i + 1]}" for i in range(0, len(v) - 1, 2))
        return d + ("Z" if tag == "polygon" else "")
    return ""


def _outline(contours, m=IDENTITY):
    ol = Outline()
    for pts, closed in contours:
        c = Contour()
        for x, y, fl in pts:
            c.points.append(_apply(m, x, y))
            c.flags.append(fl)
        c.closed = closed
        ol.contours.append(c)
    return ol


def _bbox(contours):
    xs = [p[0] for c in contours for p in c[0]]
    ys = [p[1] for c in contours for p in c[0]]
    return (min(xs), min(ys), max(xs), max(ys)) if xs else (0.0, 0.0, 0.0, 0.0)


def _alpha(opacity: float, base_a: int = 255) -> int:
    """base_color.a *= opacity, ColorF::to_u8 (svg/src/lib.rs:360-363)."""
    import numpy as np
    a = np.float32(np.float32(base_a) * np.float32(1.0 / 255.0)) * np.float32(opacity)
    return int(np.rint(np.float32(a) * np.float32(255.0)))


@dataclass
class SVGScene:
    """The result of load_svg: the scene and what the document used that this
    front-end does not draw (BuildResultFlags, svg/src/lib.rs:47-60)."""
    scene: Scene
    unsupported: set
    stroke_count: int = 0
    fill_count: int = 0


def _url_id(v):
    m = re.match(r"\s*url\(\s*#([^)\s]+)\s*\)", v or "")
    return m.group(1) if m else None


def _gradient_defs(root):
    """id -> gradient element attributes and stops, with xlink:href inheritance."""
    raw = {}
    for el in root.iter():
        if _tag(el) in ("linearGradient", "radialGradient") and el.get("id"):
            stops = []
            for st in el:
                if _tag(st) != "stop":
                    continue
                sa = _style(st)
                off = sa.get("offset", "0").strip()
                off = float(off[:-1]) / 100.0 if off.endswith("%") else _length(off)
                stops.append((min(1.0, max(0.0, off)), parse_color(sa.get("stop-color", "black")) or (0, 0, 0),
                              float(sa.get("stop-opacity", "1"))))
            href = el.get("{http://www.w3.org/1999/xlink}href") or el.get("href")
            raw[el.get("id")] = (_tag(el), dict(el.attrib), stops, href[1:] if href and href.startswith("#") else None)
    out = {}
    for gid, (tag, attrs, stops, href) in raw.items():
        if not stops and href in raw:
            stops = raw[href][2]
            attrs = {**raw[href][1], **attrs}
        out[gid] = (tag, attrs, stops)
    return out


def _make_gradient(gdef, m, bbox):
    """Gradient in scene space for a path with local bbox (usvg resolves
    objectBoundingBox units; svg/src/lib.rs:190-262 builds the gradient)."""
    tag, a, stops = gdef

    def coord(k, default, extent, origin):
        v = a.get(k, default)
        frac = v.strip().endswith("%")
        x = float(v.strip()[:-1]) / 100.0 if frac else _length(v)
        return x

    obb = a.get("gradientUnits", "objectBoundingBox") != "userSpaceOnUse"
    if tag == "linearGradient":
        p0 = (coord("x1", "0%", 0, 0), coord("y1", "0%", 0, 0))
        p1 = (coord("x2", "100%", 0, 0), coord("y2", "0%", 0, 0))
        g = Gradient.linear(p0, p1)
    else:
        cx, cy, r = coord("cx", "50%", 0, 0), coord("cy", "50%", 0, 0), coord("r", "50%", 0, 0)
        fx, fy = coord("fx", a.get("cx", "50%"), 0, 0), coord("fy", a.get("cy", "50%"), 0, 0)
        g = Gradient.radial(((fx, fy), (cx, cy)), (0.0, r))
    spread = a.get("spreadMethod", "pad")
    for off, rgb, op in stops:
        g.add_color_stop(ColorU(*rgb, _alpha(op)), off * 0.5 if spread == "reflect" else off)
    if spread == "reflect":  # svg/src/lib.rs:245-253
        for off, rgb, op in stops:
            g.add_color_stop(ColorU(*rgb, _alpha(op)), 1.0 - off * 0.5)
    if spread in ("reflect", "repeat"):
        g.set_wrap(GradientWrap.REPEAT)
    t = parse_transform(a.get("gradientTransform"))
    if obb:
        x0, y0, x1, y1 = bbox
        t = _mul((x1 - x0, 0.0, 0.0, y1 - y0, x0, y0), t)
    full = _mul(m, t)
    g.apply_transform((full[0], full[2], full[1], full[3], full[4], full[5]))
    return g


def load_svg(text: str, renderer=None) -> SVGScene:
    """Parse an SVG document into a Scene.  Strokes are converted on the GPU,
    so a document with strokes needs `renderer`."""
    root = ET.fromstring(text)
    a = _style(root)
    vb = [float(v) for v in re.findall(_NUM, root.get("viewBox", ""))]
    width = _length(a.get("width"), vb[2] if len(vb) == 4 else 0.0)
    height = _length(a.get("height"), vb[3] if len(vb) == 4 else 0.0)
    m0 = IDENTITY
    if len(vb) == 4 and vb[2] > 0 and vb[3] > 0:
        s = min(width / vb[2], height / vb[3])  # preserveAspectRatio xMidYMid meet
        m0 = (s, 0.0, 0.0, s, -vb[0] * s + (width - vb[2] * s) / 2, -vb[1] * s + (height - vb[3] * s) / 2)
    grads = _gradient_defs(root)
    clips = {el.get("id"): el for el in root.iter() if _tag(el) == "clipPath" and el.get("id")}
    scene = Scene()
    scene.set_view_box(RectF(0.0, 0.0, float(width), float(height)))
    unsupported: set = set()
    items, strokes = [], []

    def paint_of(value, opacity, m, contours):
        gid = _url_id(value)
        if gid is not None:
            if gid in grads:
                return ColorU(255, 255, 255, _alpha(opacity)), _make_gradient(grads[gid], m, _bbox(contours))
            unsupported.add("non-color paint")
            return ColorU(0, 0, 0, _alpha(opacity)), None
        rgb = parse_color(value)
        return (None if rgb is None else ColorU(*rgb, _alpha(opacity))), None

    def clip_outline(cid, m):
        el = clips[cid]
        conts = []
        for kid in el.iter():
            tag = _tag(kid)
            if tag == "clipPath":
                continue
            ka = _style(kid)
            d = ka.get("d") if tag == "path" else _shape_path(tag, ka)
            if d:
                km = _mul(m, parse_transform(ka.get("transform")))
                conts += [([(*_apply(km, x, y), f) for x, y, f in pts], closed) for pts, closed in parse_path_data(d)]
        return _outline(conts)

    def walk(el, st: _State):
        tag = _tag(el)
        if tag in ("defs", "clipPath", "linearGradient", "radialGradient", "title", "desc", "metadata", "style"):
            return
        ea = _style(el)
        attrs = {**st.attrs, **{k: ea[k] for k in _INHERITED if k in ea}}
        m = _mul(st.transform, parse_transform(ea.get("transform")))
        clip = st.clip
        cid = _url_id(ea.get("clip-path"))
        if cid is not None:
            if cid in clips:
                clip = scene.push_clip_path(ClipPath(clip_outline(cid, m), clip_path=clip))
            else:
                unsupported.add("clip-path")
        if "opacity" in ea and float(ea["opacity"]) != 1.0:
            unsupported.add("opacity")
        if tag in ("svg", "g", "a", "switch"):
            for kid in el:
                walk(kid, _State(m, clip, attrs))
            return
        if tag in ("path", "rect", "circle", "ellipse", "line", "polyline", "polygon"):
            d = ea.get("d") if tag == "path" else _shape_path(tag, ea)
            contours = parse_path_data(d) if d else []
            if not contours:
                return
            fill, fg = paint_of(attrs.get("fill"), float(attrs.get("fill-opacity", "1")), m, contours)
            if fill is not None and tag not in ("line", "polyline"):
                rule = FillRule.EVEN_ODD if attrs.get("fill-rule") == "evenodd" else FillRule.WINDING
                items.append(("fill", DrawPath(_outline(contours, m), fill, rule, clip, gradient=fg)))
            stroke, sg = paint_of(attrs.get("stroke"), float(attrs.get("stroke-opacity", "1")), m, contours)
            if stroke is not None:
                style = StrokeStyle(max(_length(attrs.get("stroke-width"), 1.0), HAIRLINE_STROKE_WIDTH),
                                    {"round": LineCap.ROUND, "square": LineCap.SQUARE}.get(
                                        attrs.get("stroke-linecap"), LineCap.BUTT),
                                    {"round": LineJoin.ROUND, "bevel": LineJoin.BEVEL}.get(
                                        attrs.get("stroke-linejoin"), LineJoin.MITER),
                                    _length(attrs.get("stroke-miterlimit"), 4.0))
                dashes = _dasharray(attrs.get("stroke-dasharray"))
                if dashes:
                    strokes.append((_outline(contours), style, dashes, _length(attrs.get("stroke-dashoffset"), 0.0)))
                else:
                    strokes.append((_outline(contours), style))
                items.append(("stroke", len(strokes) - 1, stroke, sg, clip, m))
            return
        if tag in ("image", "text", "filter", "mask", "pattern", "use", "foreignObject"):
            unsupported.add(f"<{tag}>")

    walk(root, _State(m0, None, {"fill": "black"}))
    stroked = []
    if strokes:
        if renderer is None:
            raise ValueError("strokes are converted to fills on the GPU: pass a Renderer")
        stroked = renderer.stroke_to_fill(strokes)
    nf = ns = 0
    for it in items:
        if it[0] == "fill":
            scene.push_draw_path(it[1])
            nf += 1
        else:
            _, k, paint, grad, clip, m = it
            ol = stroked[k]
            for c in ol.contours:
                c.points = [_apply(m, x, y) for x, y in c.points]
            scene.push_draw_path(DrawPath(ol, paint, FillRule.WINDING, clip, gradient=grad))
            ns += 1
    return SVGScene(scene, unsupported, ns, nf)
