"""The SVG front-end on the CPU: path data, transforms, colours and shapes,
and whole documents (the reference's tiger asset when present), with strokes
converted by the oracle's stroker standing in for the GPU."""
import os

import numpy as np
import pytest

import pathfinder_gb300 as pf
from pathfinder_gb300.stroke import StrokeBatch, outlines_from_buffers
from pathfinder_gb300.svg import load_svg, parse_color, parse_path_data, parse_transform
from tests import svgdocs

# The reference's tiger asset, from the checkout named by $PATHFINDER_REFERENCE
# (the test that draws it is skipped when the variable or the file is absent).
TIGER = os.path.join(os.environ.get("PATHFINDER_REFERENCE", ""), "resources/svg/Ghostscript_Tiger.svg")


class OracleStroker:
    """The oracle's OutlineDash and OutlineStrokeToFill in place of
    PFCUDAStrokeToFill(Dashed) (CPU tests)."""

    def stroke_to_fill(self, items):
        import oracle
        b = StrokeBatch(items)
        if not b.dashed:
            return outlines_from_buffers(*oracle.stroke(b.desc())[:4])
        pts, flags, cs, closed, os_, _ = oracle.dash(b.desc(), b.dash_desc())
        dashed = outlines_from_buffers(pts, flags, cs, os_, closed)
        b2 = StrokeBatch([(ol, it[1]) for ol, it in zip(dashed, items)])
        return outlines_from_buffers(*oracle.stroke(b2.desc())[:4])


def test_path_data_commands():
    cs = parse_path_data("M10 10 h20 v20 h-20 z m5 5 l3 3 q4 0 4 4 t2 2 c1 1 2 2 3 3 s4 4 5 5 "
                         "a5 5 0 0 1 10 0 L0 0")
    assert len(cs) == 2 and cs[0][1] and not cs[1][1]
    assert cs[0][0] == [(10, 10, 0), (30, 10, 0), (30, 30, 0), (10, 30, 0)]
    pts = cs[1][0]
    assert pts[0][:2] == (15, 15) and pts[1][:2] == (18, 18)
    # the quadratic q4 0 4 4 from (18,18) as a cubic: control points at 2/3
    assert np.allclose(pts[2][:2], (18 + 8 / 3, 18)) and pts[2][2] == 1 and pts[3][2] == 2
    assert pts[-1][:2] == (0, 0)
    # an arc ends exactly at its end point, as cubics
    arc = parse_path_data("M0 0 A10 10 0 0 1 20 0")[0][0]
    assert arc[-1][:2] == (20, 0) and all(abs(np.hypot(x - 10, y) - 10) < 1e-9 for x, y, f in arc if f == 0)


def test_transforms_and_colours():
    m = parse_transform("translate(10 20) scale(2) rotate(90)")
    x, y = m[0] * 1 + m[2] * 0 + m[4], m[1] * 1 + m[3] * 0 + m[5]
    assert np.allclose((x, y), (10, 22))
    assert parse_color("#f0a") == (255, 0, 170) and parse_color("rgb(10, 20, 30)") == (10, 20, 30)
    assert parse_color("none") is None and parse_color("navy") == (0, 0, 128)


def test_document_structure(built):
    r = load_svg(svgdocs.document(0), OracleStroker())
    s = r.scene
    assert r.stroke_count == 26 and not r.unsupported
    assert len(s.draw_paths) == r.fill_count + r.stroke_count
    assert len(s.clip_paths) >= 1 and len(s.gradients) >= 1
    assert s.width == 256 and s.height == 192
    with pytest.raises(ValueError):
        load_svg(svgdocs.document(0))  # strokes need a renderer


def test_document_renders(built):
    import oracle
    r = load_svg(svgdocs.document(1), OracleStroker())
    img, _ = oracle.OracleFrame(r.scene).render(r.scene.width, r.scene.height)
    assert (img[..., 3] > 0).mean() > 0.05


@pytest.mark.skipif(not os.path.exists(TIGER), reason="the reference's tiger asset is not on this machine")
def test_tiger(built):
    """The reference's tiger (resources/svg/Ghostscript_Tiger.svg): 138 <path>s,
    130 fills and 52 strokes drawn; the image is mostly covered."""
    import oracle
    r = load_svg(open(TIGER).read(), OracleStroker())
    assert (r.fill_count, r.stroke_count) == (130, 52) and not r.unsupported
    img, _ = oracle.OracleFrame(r.scene).render(r.scene.width, r.scene.height)
    assert (img[..., 3] > 0).mean() > 0.6


def test_dasharray_attribute():
    from pathfinder_gb300.svg import _dasharray
    assert _dasharray(None) is None and _dasharray("none") is None
    assert _dasharray("4 2") == [4.0, 2.0]
    assert _dasharray("5,1,2") == [5.0, 1.0, 2.0, 5.0, 1.0, 2.0]  # odd counts repeat
    assert _dasharray("3 -1") is None and _dasharray("0 0") is None


def test_dashed_strokes(built):
    """A dashed stroke becomes several closed pieces (each dash stroked as an
    open contour); without a pattern, one ring pair."""
    doc = ('<svg xmlns="http://www.w3.org/2000/svg" width="64" height="64">'
           '<g stroke="black" stroke-width="2" fill="none">'
           '<path d="M4 8 H60" stroke-dasharray="6 4" stroke-dashoffset="1"/>'
           '<path d="M4 20 H60"/></g></svg>')
    out = load_svg(doc, OracleStroker())
    assert out.stroke_count == 2 and "stroke-dasharray" not in out.unsupported
    sc = out.scene
    dp = sc.draw_paths
    assert int(dp[1]["contour_count"]) == 1 and int(dp[0]["contour_count"]) >= 5
    c0 = int(dp[0]["first_contour"])
    a, b = int(sc.contour_starts[c0]), int(sc.contour_starts[c0 + int(dp[0]["contour_count"])])
    ys = sc.points[a:b, 1]
    assert ys.min() == 7 and ys.max() == 9
