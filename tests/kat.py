"""Hand-built scenes for the tiler known-answer cases."""
import pathfinder_gb300 as pf


def rect_scene(x0, y0, x1, y1, w=64, h=64, rule=pf.FillRule.WINDING, paint=pf.ColorU(255, 0, 0, 255)):
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, w, h))
    c = pf.Contour().push_endpoint(x0, y0).push_endpoint(x1, y0).push_endpoint(x1, y1).push_endpoint(x0, y1)
    s.push_draw_path(pf.DrawPath(pf.Outline([c]), paint, rule))
    return s


def poly_scene(points, w=64, h=64, rule=pf.FillRule.WINDING, paint=pf.ColorU(255, 0, 0, 255)):
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, w, h))
    c = pf.Contour()
    for x, y in points:
        c.push_endpoint(x, y)
    s.push_draw_path(pf.DrawPath(pf.Outline([c]), paint, rule))
    return s
