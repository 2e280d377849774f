"""Small seeded scenes for the differentiable-rendering tests: closed cubic
blobs, optionally with holes, clip paths, even-odd rules and quadratic or
line segments."""
import numpy as np

import pathfinder_gb300 as pf


def blob_points(rng, cx, cy, r, k=5, jitter=0.1):
    """Closed cubic blob: k on-curve points around (cx, cy), control points
    near the chords."""
    ang = np.sort(rng.uniform(0, 2 * np.pi, k))
    v = [np.array([cx + r * np.cos(a), cy + r * np.sin(a)]) for a in ang]
    pts = [tuple(v[0])]
    for i in range(k):
        a, b = v[i], v[(i + 1) % k]
        c0 = a + (b - a) / 3 + rng.normal(0, r * jitter, 2)
        c1 = a + 2 * (b - a) / 3 + rng.normal(0, r * jitter, 2)
        pts += [tuple(c0), tuple(c1), tuple(b)]
    return pts


def cubic_contour(pts, reverse=False):
    """Closed chain of cubics through pts = [v0, c, c, v1, ..., c, c, v0]
    (reversed: the same chain traversed backwards)."""
    if reverse:
        pts = pts[::-1]
    c = pf.Contour()
    c.push_endpoint(*pts[0])
    for i in range(1, len(pts) - 2, 3):
        c.push_cubic(*pts[i], *pts[i + 1], *pts[i + 2])
    c.close()
    return c


def mixed_contour(rng, cx, cy, r, k=9):
    """Star-like contour of lines, quadratics and cubics."""
    c = pf.Contour()
    ang = np.sort(rng.uniform(0, 2 * np.pi, k))
    v = [(cx + r * rng.uniform(0.6, 1.0) * np.cos(a), cy + r * rng.uniform(0.6, 1.0) * np.sin(a)) for a in ang]
    c.push_endpoint(*v[0])
    for i in range(1, k + 1):
        b = v[i % k]
        kind = i % 3
        if kind == 0:
            c.push_endpoint(*b)
        elif kind == 1:
            m = ((v[i - 1][0] + b[0]) / 2 + rng.normal(0, 3), (v[i - 1][1] + b[1]) / 2 + rng.normal(0, 3))
            c.push_quadratic(*m, *b)
        else:
            a = v[i - 1]
            c.push_cubic(a[0] + (b[0] - a[0]) / 3 + rng.normal(0, 2), a[1] + (b[1] - a[1]) / 3 + rng.normal(0, 2),
                         a[0] + 2 * (b[0] - a[0]) / 3 + rng.normal(0, 2), a[1] + 2 * (b[1] - a[1]) / 3 + rng.normal(0, 2),
                         *b)
    c.close()
    return c


def blobs(W=96, H=96, n=6, seed=0, even_odd=False, alpha=(0.3, 0.95), holes=False, edge=False):
    """n cubic blobs on a W x H canvas (edge=True lets them cross the canvas edge)."""
    rng = np.random.default_rng(seed)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    rule = pf.FillRule.EVEN_ODD if even_odd else pf.FillRule.WINDING
    for _ in range(n):
        lo, hi = (-0.1, 1.1) if edge else (0.25, 0.75)
        cx, cy = rng.uniform(lo * W, hi * W), rng.uniform(lo * H, hi * H)
        r = rng.uniform(0.1, 0.25) * min(W, H)
        contours = [cubic_contour(blob_points(rng, cx, cy, r))]
        if holes:
            contours.append(cubic_contour(blob_points(rng, cx, cy, 0.4 * r), reverse=not even_odd))
        a = int(round(255 * rng.uniform(*alpha)))
        s.push_draw_path(pf.DrawPath(pf.Outline(contours), pf.ColorU(255, 255, 255, a), rule))
    return s


def mixed(W=96, H=96, n=5, seed=0):
    """Paths of lines, quadratics and cubics, one of them clipped by a clip path."""
    rng = np.random.default_rng(seed)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    clip = s.push_clip_path(pf.ClipPath(pf.Outline([cubic_contour(blob_points(rng, W / 2, H / 2, 0.35 * W))]),
                                        pf.FillRule.WINDING))
    for i in range(n):
        c = mixed_contour(rng, rng.uniform(0.3 * W, 0.7 * W), rng.uniform(0.3 * H, 0.7 * H), 0.22 * W)
        a = int(round(255 * rng.uniform(0.4, 0.9)))
        s.push_draw_path(pf.DrawPath(pf.Outline([c]), pf.ColorU(255, 255, 255, a), pf.FillRule.WINDING,
                                     clip_path=clip if i == 0 else None))
    return s
