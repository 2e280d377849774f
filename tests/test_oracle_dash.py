"""The oracle's restatement of OutlineDash (content/src/dash.rs:18-152) against
cases worked out by hand from the reference's code.

What the hand derivations follow: DashState::new (:124-145) reduces the
offset modulo the pattern's sum, skips the whole dashes it covers and starts
the distance left at what remains of the offset (so an offset of 0 starts
with an empty "on" dash); ContourDash::dash (:73-113) cuts a segment at
t = distance left / chord length (time_for_distance, segment.rs:251-254),
pushes the "on" pieces with Contour::push_segment (both end points of every
piece, outline.rs:576-600) and ends the dash contour when the distance left
drops below 1e-4; the open dash contour carries across contours, and
into_outline (:52-57) keeps the last one when it is "on".  The cut points
below are exact in single precision (each product rounds back onto the
integer or half it approximates)."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from pathfinder_gb300.stroke import StrokeBatch

CP0, CP1 = 1, 2


def _dash(items):
    import oracle
    b = StrokeBatch([(ol, None, dashes, offset) for ol, dashes, offset in items])
    return oracle.dash(b.desc(), b.dash_desc())


def _poly(*pts, closed=False):
    c = pf.Contour()
    for p in pts:
        c.push_endpoint(*p)
    if closed:
        c.close()
    return c


def _contours(pts, cs):
    return [pts[cs[i]:cs[i + 1]].tolist() for i in range(len(cs) - 1)]


def test_line_offset_zero_starts_with_an_empty_dash(built):
    """(0,0)-(8,0), dashes [2, 2], offset 0: cut at t = 0 (an empty "on" dash),
    then off to 2 (t = 2/8), on to 4 (t = 2/6), off to 6 (t = 2/4), on to 8
    (t = 2/2 = 1: the whole rest, no cut)."""
    pts, flags, cs, closed, os_, lim = _dash([(pf.Outline([_poly((0, 0), (8, 0))]), [2, 2], 0.0)])
    assert not lim
    assert _contours(pts, cs) == [[[0, 0], [0, 0]], [[2, 0], [4, 0]], [[6, 0], [8, 0]]]
    assert flags.tolist() == [0] * 6 and closed.tolist() == [0, 0, 0] and os_.tolist() == [0, 3]


def test_offset_skips_whole_dashes(built):
    """Offset 3 with [2, 2]: 3 mod 4 = 3 covers the first dash, leaving 1 of
    the "off" dash: off to 1, on to 3 (t = 2/7), off to 5 (t = 2/5), on to 7
    (t = 2/3), and the last 1 is off."""
    pts, _, cs, _, _, _ = _dash([(pf.Outline([_poly((0, 0), (8, 0))]), [2, 2], 3.0)])
    assert _contours(pts, cs) == [[[1, 0], [3, 0]], [[5, 0], [7, 0]]]


def test_closed_square_dashes_around_corners(built):
    """A closed 4x4 square with [6, 2]: the closing segment is dashed too, and
    a dash over a corner is one contour holding both pieces (the corner point
    twice)."""
    sq = _poly((0, 0), (4, 0), (4, 4), (0, 4), closed=True)
    pts, _, cs, closed, _, _ = _dash([(pf.Outline([sq]), [6, 2], 0.0)])
    assert _contours(pts, cs) == [[[0, 0], [0, 0]],
                                  [[2, 0], [4, 0], [4, 0], [4, 4]],
                                  [[2, 4], [0, 4], [0, 4], [0, 0]]]
    assert closed.tolist() == [0, 0, 0]


def test_dash_carries_across_contours(built):
    """Two open contours, [3, 1], offset 0.5: the "on" dash begun at the end
    of the first contour continues on the second (its from point follows the
    first's last), and the last dash is kept by into_outline."""
    ol = pf.Outline([_poly((0, 0), (2, 0)), _poly((10, 0), (14, 0))])
    pts, _, cs, _, os_, _ = _dash([(ol, [3, 1], 0.5)])
    assert _contours(pts, cs) == [[[0, 0], [0.5, 0]],
                                  [[1.5, 0], [2, 0], [10, 0], [12.5, 0]],
                                  [[13.5, 0], [14, 0]]]
    assert os_.tolist() == [0, 3]


def test_whole_curve_stays_quadratic(built):
    """A line then a quadratic under one long dash: after the empty first dash
    and the 1-long gap (cut at t = 1/10), the rest of the line and the whole
    quadratic are pushed as they are (3 points, control flag on the middle)."""
    c = _poly((-10, 0), (0, 0))
    c.push_quadratic(4, 4, 8, 0)
    pts, flags, cs, _, _, _ = _dash([(pf.Outline([c]), [100, 1], 0.0)])
    assert _contours(pts, cs) == [[[-10, 0], [-10, 0]], [[-9, 0], [0, 0], [0, 0], [4, 4], [8, 0]]]
    assert flags.tolist() == [0, 0, 0, 0, 0, CP0, 0]


def test_cut_curve_becomes_cubic(built):
    """A quadratic cut by a dash is split as a cubic (Segment::split through
    to_cubic): both pieces carry two control points.  The cut at t = 1/8 lies
    on the curve x = 8t, y = 8t(1-t)."""
    c = _poly((0, 0))
    c.push_quadratic(4, 4, 8, 0)
    pts, flags, cs, _, _, _ = _dash([(pf.Outline([c]), [100, 1], 0.0)])
    assert len(cs) == 3
    first, second = _contours(pts, cs)
    assert first == [[0, 0]] * 4  # the empty first dash: a degenerate cubic at t = 0
    assert flags.tolist() == [0, CP0, CP1, 0] * 2
    assert second[-1] == [8, 0]
    assert np.allclose(second[0], [1.0, 0.875], atol=1e-6)


def test_empty_pattern_passes_the_outline_through(built):
    sq = _poly((0, 0), (4, 0), (4, 4), closed=True)
    ol = pf.Outline([sq, _poly((9, 9), (10, 10))])
    pts, _, cs, closed, os_, _ = _dash([(ol, [], 0.0), (pf.Outline([_poly((0, 0), (8, 0))]), [2, 2], 0.0)])
    assert _contours(pts, cs)[:2] == [[[0, 0], [4, 0], [4, 4]], [[9, 9], [10, 10]]]
    assert closed.tolist()[:2] == [1, 0]
    assert os_.tolist() == [0, 2, 5]


def test_zero_length_dashes_give_dots(built):
    """[0, 2]: every "on" dash is empty, a two-point contour at each cut (the
    dots that round caps turn into discs)."""
    pts, _, cs, _, _, _ = _dash([(pf.Outline([_poly((0, 0), (8, 0))]), [0, 2], 0.0)])
    cont = _contours(pts, cs)
    assert [c[0] for c in cont] == [[0, 0], [2, 0], [4, 0], [6, 0]]
    assert all(c[0] == c[1] for c in cont)
