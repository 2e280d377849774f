"""The oracle's stroke-to-fill restatement (content/src/stroke.rs) against
cases worked out by hand from the reference's code, and properties of its
output (area of stroked lines and rings through the FP64 coverage)."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from pathfinder_gb300.stroke import LineCap, LineJoin, StrokeBatch, StrokeStyle, outlines_from_buffers


def _line(*pts, closed=False):
    c = pf.Contour()
    for p in pts:
        c.push_endpoint(*p)
    if closed:
        c.close()
    return pf.Outline([c])


def _stroke(items):
    import oracle
    b = StrokeBatch(items)
    return oracle.stroke(b.desc())


def test_butt_line_is_a_rectangle(built):
    """(0,0)-(10,0), width 2, butt caps: offset_forward gives the y = -1 side,
    offset_backward the y = +1 side (stroke.rs:208-230), no caps."""
    pts, flags, cs, os_, lim = _stroke([(_line((0, 0), (10, 0)), StrokeStyle(2.0, LineCap.BUTT))])
    assert not lim and list(cs) == [0, 4] and list(os_) == [0, 1]
    assert pts.tolist() == [[0, -1], [10, -1], [10, 1], [0, 1]]
    assert flags.tolist() == [0, 0, 0, 0]


def test_square_caps(built):
    """add_cap Square (stroke.rs:175-186): p2 = p1 + g w/2, p3 = p2 + g.yx (-w, w),
    p4 = p3 - g w/2, after each pass."""
    pts, _, cs, _, _ = _stroke([(_line((0, 0), (10, 0)), StrokeStyle(2.0, LineCap.SQUARE))])
    assert pts.tolist() == [[0, -1], [10, -1], [11, -1], [11, 1], [10, 1],
                            [10, 1], [0, 1], [-1, 1], [-1, -1], [0, -1]]


def test_closed_square_miters(built):
    """A closed 10x10 square, width 2, miter joins: the forward contour is the
    outer square with a miter point at each corner (add_join Miter,
    stroke.rs:424-436), the closing join included (push_stroked_contour,
    :135-149); the backward contour lies on the inner square."""
    sq = _line((0, 0), (10, 0), (10, 10), (0, 10), closed=True)
    pts, _, cs, _, _ = _stroke([(sq, StrokeStyle(2.0, LineCap.BUTT, LineJoin.MITER, 10.0))])
    assert len(cs) == 3
    outer = pts[cs[0]:cs[1]]
    # the miter points come out of intersection_t in single precision (10.999999)
    assert np.allclose(outer, [[0, -1], [10, -1], [11, -1], [11, 0], [11, 10], [11, 11], [10, 11], [0, 11],
                               [-1, 11], [-1, 10], [-1, 0], [-1, -1]], atol=1e-5, rtol=0)
    inner = pts[cs[1]:cs[2]]
    assert np.all((np.isclose(inner[:, 0], 1) | np.isclose(inner[:, 0], 9) |
                   np.isclose(inner[:, 1], 1) | np.isclose(inner[:, 1], 9)))
    bevel = _stroke([(sq, StrokeStyle(2.0, LineCap.BUTT, LineJoin.BEVEL))])[0]
    assert len(bevel) == 16  # no join points


def test_round_join_and_cap_points_on_circles(built):
    """Round joins and caps push cubic arcs of radius w/2 around the join point
    or the line end (push_arc_from_unit_chord, outline.rs:630-669): their end
    points lie on the circle."""
    ol = _line((0, 0), (20, 0), (20, 20))
    pts, flags, cs, _, _ = _stroke([(ol, StrokeStyle(4.0, LineCap.ROUND, LineJoin.ROUND))])
    on = pts[flags == 0]
    d_join = np.hypot(on[:, 0] - 20, on[:, 1] - 0)
    d_end = np.hypot(on[:, 0] - 20, on[:, 1] - 20)
    d_start = np.hypot(on[:, 0], on[:, 1])
    near = np.minimum(np.minimum(np.abs(d_join - 2), np.abs(d_end - 2)), np.abs(d_start - 2))
    assert near.max() < 1e-4


def _coverage_area(outline, W, H):
    import oracle
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    s.push_draw_path(pf.DrawPath(outline, pf.ColorU(255, 255, 255, 255)))
    _, f = oracle.OracleFrame(s).render(W, H)
    return f[..., 3].sum()


@pytest.mark.parametrize("cap,extra", [(LineCap.BUTT, 0.0), (LineCap.SQUARE, 2 * 1.5 * 3), (LineCap.ROUND, np.pi * 1.5 ** 2)])
def test_stroked_line_area(built, cap, extra):
    """Area of a stroked diagonal line: length x width, plus the caps."""
    ol = _line((10.3, 12.1), (50.7, 41.9))
    pts, flags, cs, os_, _ = _stroke([(ol, StrokeStyle(3.0, cap))])
    out = outlines_from_buffers(pts, flags, cs, os_)[0]
    length = np.hypot(40.4, 29.8)
    assert abs(_coverage_area(out, 64, 64) - (length * 3.0 + extra)) < 0.02 * (length * 3.0)


def test_stroked_ring_area(built):
    """A closed circle-like contour of radius 20 stroked at width 4: the ring's
    area 2 pi r w, from the forward and backward contours filled nonzero."""
    c = pf.Contour()
    k = 8
    r = 20.0
    for i in range(k):
        a0, a1 = 2 * np.pi * i / k, 2 * np.pi * (i + 1) / k
        h = 4.0 / 3.0 * np.tan((a1 - a0) / 4)
        p0 = np.array([np.cos(a0), np.sin(a0)]) * r + 32
        p3 = np.array([np.cos(a1), np.sin(a1)]) * r + 32
        c0 = p0 + h * r * np.array([-np.sin(a0), np.cos(a0)])
        c1 = p3 - h * r * np.array([-np.sin(a1), np.cos(a1)])
        if i == 0:
            c.push_endpoint(*p0)
        c.push_cubic(*c0, *c1, *p3)
    c.close()
    pts, flags, cs, os_, lim = _stroke([(pf.Outline([c]), StrokeStyle(4.0, line_join=LineJoin.ROUND))])
    assert not lim and len(cs) == 3
    out = outlines_from_buffers(pts, flags, cs, os_)[0]
    assert abs(_coverage_area(out, 64, 64) - 2 * np.pi * r * 4.0) < 0.01 * 2 * np.pi * r * 4.0


def test_open_contour_edge_cases(built):
    """Empty, single-point and coincident-point contours stroke without error;
    each contour still yields its contour(s)."""
    c0 = pf.Contour()
    c1 = pf.Contour().push_endpoint(5, 5)
    c2 = pf.Contour().push_endpoint(5, 5).push_endpoint(5, 5).push_endpoint(5, 5)
    c3 = pf.Contour().push_endpoint(1, 1).close()
    ol = pf.Outline([c0, c1, c2, c3])
    pts, flags, cs, os_, _ = _stroke([(ol, StrokeStyle(2.0, LineCap.ROUND, LineJoin.ROUND))])
    assert list(os_) == [0, 5]  # open: 1 each, closed: 2


def test_huge_input_is_bounded(built):
    import time
    c = pf.Contour()
    c.push_endpoint(0, 0)
    c.push_cubic(1e30, -1e30, -1e30, 1e30, 50, 50)
    t = time.time()
    _, _, _, _, lim = _stroke([(pf.Outline([c]), StrokeStyle(3.0))])
    assert lim and time.time() - t < 60
