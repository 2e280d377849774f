"""Seeded outlines to stroke: open and closed contours of lines, quadratics and
cubics, sharp and shallow corners, tiny and coincident segments, every cap and
join."""
import numpy as np

import pathfinder_gb300 as pf
from pathfinder_gb300.stroke import LineCap, LineJoin, StrokeStyle


def random_contour(rng, cx, cy, r, k, closed):
    c = pf.Contour()
    ang = np.sort(rng.uniform(0, 2 * np.pi, k)) if closed else rng.uniform(0, 2 * np.pi, k)
    pts = [(cx + r * rng.uniform(0.3, 1.0) * np.cos(a), cy + r * rng.uniform(0.3, 1.0) * np.sin(a)) for a in ang]
    c.push_endpoint(*pts[0])
    for i in range(1, k):
        x, y = pts[i]
        kind = rng.integers(0, 4)
        px, py = pts[i - 1]
        if kind == 0:
            c.push_quadratic((px + x) / 2 + rng.normal(0, r / 3), (py + y) / 2 + rng.normal(0, r / 3), x, y)
        elif kind == 1:
            c.push_cubic(px + rng.normal(0, r / 3), py + rng.normal(0, r / 3), x + rng.normal(0, r / 3),
                         y + rng.normal(0, r / 3), x, y)
        elif kind == 2 and i + 1 < k:
            c.push_endpoint(px + 0.003, py)  # a tiny segment
            c.push_endpoint(x, y)
        else:
            c.push_endpoint(x, y)
    if closed:
        c.close()
    return c


def stroke_items(seed=0, n=40, W=256, H=256):
    rng = np.random.default_rng(seed)
    items = []
    for i in range(n):
        ol = pf.Outline()
        for _ in range(int(rng.integers(1, 4))):
            ol.contours.append(random_contour(rng, rng.uniform(0, W), rng.uniform(0, H), rng.uniform(5, 60),
                                              int(rng.integers(2, 9)), bool(rng.integers(0, 2))))
        st = StrokeStyle(float(rng.choice([0.5, 1.0, 2.5, 6.0, 13.0])), LineCap(int(rng.integers(0, 3))),
                         LineJoin(int(rng.integers(0, 3))), float(rng.choice([1.5, 4.0, 10.0])))
        items.append((ol, st))
    # edge cases: empty, single point, coincident points, a straight back-and-forth
    e = pf.Outline([pf.Contour(), pf.Contour().push_endpoint(3, 3),
                    pf.Contour().push_endpoint(5, 5).push_endpoint(5, 5).push_endpoint(5, 5),
                    pf.Contour().push_endpoint(1, 1).close(),
                    pf.Contour().push_endpoint(10, 10).push_endpoint(40, 10).push_endpoint(10, 10)])
    items.append((e, StrokeStyle(4.0, LineCap.ROUND, LineJoin.ROUND)))
    items.append((e, StrokeStyle(4.0, LineCap.SQUARE, LineJoin.MITER, 4.0)))
    return items
