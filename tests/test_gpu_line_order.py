"""Plain frames flatten in one pass: each block of the flattening kernel takes
its range of lines with one atomic, so the frame's line order depends on the
schedule.  Frames run for record read-back flatten in depth-first order (count,
scan, emit).  No output may depend on which: fill counts, raw masks (integer
sums of the same fills) and resolved tile coverage of a plain frame must equal
those of the ordered frame bit for bit."""
import numpy as np
import pytest

import pathfinder_gb300 as pf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("workload, seed, scale", [(pf.PF_SCENE_SVG_4K, 2, 0.05), (pf.PF_SCENE_CUBIC_1K, 3, 1.0),
                                                    (pf.PF_SCENE_EDGE_CASES, 1, 1.0)])
def test_plain_frame_equals_ordered_frame(renderer, workload, seed, scale):
    s = pf.generate_scene(workload, seed=seed, scale=scale)
    renderer.render(s)
    st_plain = renderer.stats()
    a_plain, t_plain = renderer.read_masks()  # from the plain frame's fills
    renderer.read_records(s)  # re-runs the frame with its lines in depth-first order
    st_ord = renderer.stats()
    a_ord, t_ord = renderer.read_masks()
    for k in ("line_count", "fill_count", "tile_count", "alpha_tile_count", "visible_tile_count"):
        assert getattr(st_plain, k) == getattr(st_ord, k), k
    assert st_plain.line_count > 0
    assert np.array_equal(a_plain, a_ord)
    assert np.array_equal(t_plain, t_ord)


def big_curve_scene(n_paths=400, k=80, W=1024, H=1024, seed=0):
    """Closed paths of large cubics: many more lines than two per segment,
    past the line capacity an upload reserves (2 per segment, at least
    65,536), so the first frame regrows it."""
    rng = np.random.default_rng(seed)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    for _ in range(n_paths):
        cx, cy, r = rng.uniform(0, W), rng.uniform(0, H), rng.uniform(200, 600)
        a = np.sort(rng.uniform(0, 2 * np.pi, k))
        pts = [(cx + r * np.cos(t), cy + r * np.sin(t)) for t in a]
        c = pf.Contour().push_endpoint(*pts[0])
        for i in range(1, k):
            (px, py), (x, y) = pts[i - 1], pts[i]
            c.push_cubic(px + rng.normal(0, r), py + rng.normal(0, r), x + rng.normal(0, r), y + rng.normal(0, r), x, y)
        c.close()
        s.push_draw_path(pf.DrawPath(pf.Outline([c]), pf.ColorU(*[int(v) for v in rng.integers(0, 256, 3)], 60)))
    return s


def test_line_capacity_regrows(renderer):
    """A frame whose lines overflow the reserved line array (both of the
    one-pass flattening's ranges) regrows it and renders the ordered frame's
    coverage."""
    import oracle
    from tests.parity import compare_images
    s = big_curve_scene()
    segs = len(s.points)  # an upper bound of the segment count
    img = renderer.render(s)
    st = renderer.stats()
    assert st.status == 0 and st.line_count > max(65536, 2 * segs)
    a_plain, t_plain = renderer.read_masks()
    renderer.read_records(s)
    a_ord, t_ord = renderer.read_masks()
    assert renderer.stats().line_count == st.line_count
    assert np.array_equal(a_plain, a_ord) and np.array_equal(t_plain, t_ord)
    ora, _ = oracle.OracleFrame(s).render(1024, 1024)
    compare_images(img, ora)
