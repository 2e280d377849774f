"""Seeded scenes with paint effects (gradients and blend modes) for the
oracle and GPU parity tests."""
import numpy as np

import pathfinder_gb300 as pf


def blob(rng, cx, cy, r, k=10, quad=True):
    c = pf.Contour()
    ang = np.sort(rng.uniform(0, 2 * np.pi, k))
    pts = [(cx + r * rng.uniform(0.7, 1.0) * np.cos(a), cy + r * rng.uniform(0.7, 1.0) * np.sin(a)) for a in ang]
    c.push_endpoint(*pts[0])
    for i in range(1, k + 1):
        x, y = pts[i % k]
        if quad and i % 2:
            px, py = pts[i - 1]
            c.push_quadratic((px + x) / 2 + rng.normal(0, 3), (py + y) / 2 + rng.normal(0, 3), x, y)
        else:
            c.push_endpoint(x, y)
    c.close()
    return pf.Outline([c])


def rect(x0, y0, x1, y1):
    c = pf.Contour()
    c.push_endpoint(x0, y0)
    c.push_endpoint(x1, y0)
    c.push_endpoint(x1, y1)
    c.push_endpoint(x0, y1)
    c.close()
    return pf.Outline([c])


def color(rng, a=None):
    return pf.ColorU(int(rng.integers(0, 256)), int(rng.integers(0, 256)), int(rng.integers(0, 256)),
                     int(rng.integers(60, 256)) if a is None else a)


def stops(g, rng, n=4, opaque=False):
    for _ in range(n):
        g.add_color_stop(color(rng, 255 if opaque else None), float(rng.uniform(0, 1)))
    return g


def linear(rng, W, H, wrap=pf.GradientWrap.CLAMP, opaque=False):
    g = pf.Gradient.linear((rng.uniform(0, W), rng.uniform(0, H)), (rng.uniform(0, W), rng.uniform(0, H)))
    g.set_wrap(wrap)
    return stops(g, rng, opaque=opaque)


def radial(rng, W, H, wrap=pf.GradientWrap.CLAMP, focal=False, opaque=False):
    """Concentric, or with the first circle inside the second (no cone edge)."""
    cx, cy = rng.uniform(0.3 * W, 0.7 * W), rng.uniform(0.3 * H, 0.7 * H)
    r1 = rng.uniform(0.3, 0.6) * min(W, H)
    if focal:
        off = rng.uniform(0.05, 0.3) * r1
        a = rng.uniform(0, 2 * np.pi)
        g = pf.Gradient.radial(((cx + off * np.cos(a), cy + off * np.sin(a)), (cx, cy)), (0.05 * r1, r1))
    else:
        g = pf.Gradient.radial((cx, cy), (0.0, r1))
    g.set_wrap(wrap)
    return stops(g, rng, opaque=opaque)


def backdrop(s, rng, W, H, n=4):
    """Opaque and translucent solid blobs for the blend modes to act on."""
    s.push_draw_path(pf.DrawPath(rect(0.1 * W, 0.15 * H, 0.7 * W, 0.8 * H), color(rng, 255)))
    for _ in range(n):
        s.push_draw_path(pf.DrawPath(blob(rng, rng.uniform(0.2 * W, 0.8 * W), rng.uniform(0.2 * H, 0.8 * H),
                                          rng.uniform(0.15, 0.35) * min(W, H), 9, rng), color(rng)))


def blend_scene(mode, seed=0, W=112, H=96, gradient=False):
    """A backdrop, then two paths drawn with ``mode`` (one solid, one with a
    gradient when asked), then a SrcOver path on top."""
    rng = np.random.default_rng(seed * 131 + int(mode))
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    backdrop(s, rng, W, H)
    s.push_draw_path(pf.DrawPath(blob(rng, 0.45 * W, 0.5 * H, 0.3 * min(W, H), 11, rng), color(rng),
                                 blend_mode=int(mode)))
    g = linear(rng, W, H) if gradient else None
    s.push_draw_path(pf.DrawPath(blob(rng, 0.6 * W, 0.4 * H, 0.25 * min(W, H), 10, rng), color(rng, 230),
                                 pf.FillRule.EVEN_ODD, blend_mode=int(mode), gradient=g))
    s.push_draw_path(pf.DrawPath(blob(rng, 0.3 * W, 0.7 * H, 0.15 * min(W, H), 8, rng), color(rng)))
    return s


def gradient_scene(seed=0, W=160, H=128, clip=True):
    """Every gradient kind and wrap over a backdrop, some clipped, some opaque."""
    rng = np.random.default_rng(seed)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    backdrop(s, rng, W, H, n=2)
    c = s.push_clip_path(pf.ClipPath(blob(rng, 0.5 * W, 0.5 * H, 0.45 * min(W, H), 12, rng))) if clip else None
    grads = [linear(rng, W, H), linear(rng, W, H, pf.GradientWrap.REPEAT),
             radial(rng, W, H), radial(rng, W, H, pf.GradientWrap.REPEAT),
             radial(rng, W, H, focal=True), linear(rng, W, H, opaque=True), radial(rng, W, H, opaque=True)]
    for i, g in enumerate(grads):
        base = pf.ColorU(255, 255, 255, 255 if i >= 5 else int(rng.integers(120, 256)))
        s.push_draw_path(pf.DrawPath(blob(rng, rng.uniform(0.2 * W, 0.8 * W), rng.uniform(0.2 * H, 0.8 * H),
                                          rng.uniform(0.2, 0.4) * min(W, H), 11, rng), base,
                                     clip_path=c if (clip and i % 3 == 1) else None, gradient=g))
    # a large opaque gradient rectangle: its solid tiles occlude what lies below
    s.push_draw_path(pf.DrawPath(rect(0.55 * W, 0.05 * H, 0.98 * W, 0.6 * H), pf.ColorU(255, 255, 255, 255),
                                 gradient=grads[5]))
    return s


def image(rng, w, h, opaque=False):
    """A seeded straight-alpha RGBA8 image: smooth colour ramps with noise."""
    y, x = np.mgrid[0:h, 0:w]
    img = np.zeros((h, w, 4), np.float64)
    img[..., 0] = 255 * x / max(1, w - 1)
    img[..., 1] = 255 * y / max(1, h - 1)
    img[..., 2] = 128 + 127 * np.sin(x * 0.7 + y * 0.3)
    img[..., 3] = 255 if opaque else 60 + 195 * ((x + y) % 7) / 6
    img[..., :3] += rng.normal(0, 20, (h, w, 3))
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def pattern_scene(seed=0, W=160, H=128, filters=True):
    """Image patterns with every repeat/smoothing combination, rotated and
    scaled, with blur and colour-matrix filters, over a backdrop."""
    rng = np.random.default_rng(seed)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    backdrop(s, rng, W, H, n=2)
    k = 0
    for rx in (False, True):
        for ry in (False, True):
            for smooth in (True, False):
                p = pf.Pattern.from_image(image(rng, int(rng.integers(5, 24)), int(rng.integers(5, 24)), opaque=k % 3 == 0))
                p.repeat_x, p.repeat_y, p.smoothing = rx, ry, smooth
                a, sc = rng.uniform(0, 2 * np.pi), rng.uniform(0.6, 3.0)
                p.apply_transform((sc * np.cos(a), -sc * np.sin(a), sc * np.sin(a), sc * np.cos(a),
                                   rng.uniform(0, W), rng.uniform(0, H)))
                if filters and k % 4 == 1:
                    p.set_blur(float(rng.uniform(0.5, 3.0)), "x" if k % 8 == 1 else "y")
                elif filters and k % 4 == 3:
                    cols = np.zeros((5, 4), np.float32)
                    cols[0] = (0.3, 0.3, 0.3, 0)   # r -> greyish
                    cols[1] = (0.59, 0.59, 0.2, 0)
                    cols[2] = (0.11, 0.11, 0.8, 0)
                    cols[3] = (0, 0, 0, 1)
                    cols[4] = (0.05, -0.05, 0.1, 0)
                    p.set_color_matrix(cols)
                base = pf.ColorU(255, 255, 255, 255 if k % 2 == 0 else 190)
                s.push_draw_path(pf.DrawPath(blob(rng, rng.uniform(0.2 * W, 0.8 * W), rng.uniform(0.2 * H, 0.8 * H),
                                                  rng.uniform(0.2, 0.4) * min(W, H), 11, rng), base, pattern=p,
                                             blend_mode=int(pf.BlendMode.MULTIPLY) if k == 6 else 0))
                k += 1
    return s
