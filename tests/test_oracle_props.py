"""Size-independent properties of the oracle restatement."""
import numpy as np

import oracle
import pathfinder_gb300 as pf
from tests.kat import rect_scene


def test_thread_count_does_not_change_the_build(built):
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=2, scale=0.02)
    a, b = oracle.OracleFrame(s, threads=1), oracle.OracleFrame(s, threads=8)
    fa, ta = a.fills()
    fb, tb = b.fills()
    assert np.array_equal(fa, fb) and np.array_equal(ta, tb)
    assert np.array_equal(a.tiles()[0], b.tiles()[0])
    assert np.array_equal(a.zbuffer(), b.zbuffer())


def test_single_fill_integrates_to_its_signed_area(built):
    rng = np.random.default_rng(0)
    for _ in range(200):
        seg = rng.integers(0, 4096, 4)
        if seg[0] == seg[2]:
            continue
        m = oracle.fill_coverage(seg)
        x0, y0, x1, y1 = seg / 256.0
        # signed area of the tile below the segment: integral from x1 to x0 of (16 - y)
        expect = (x0 - x1) * (16.0 - 0.5 * (y0 + y1))
        assert abs(m.sum() - expect) < 1e-9


def test_rect_interior_is_fully_covered(built):
    fr = oracle.OracleFrame(rect_scene(5.25, 7.5, 60.75, 58.0, w=64, h=64))
    img, f64 = fr.render(64, 64)
    a = f64[..., 3]
    # interior pixels are covered; a fill that runs to a tile's right edge is
    # clamped to x = 4095/256 (builder.rs:527-529), which leaves the last
    # 1/256 px column of such a tile uncovered
    assert np.all(np.abs(a[8:58, 6:60] - 1.0) <= 1.0 / 256 + 1e-12)
    assert np.allclose(a[24:58, 6:60], 1.0)
    # outside: zero, up to the same 1/256 residue in a tile's last column
    # below an edge whose fill was clamped
    assert np.all(a[59:, :] <= 1.0 / 256 + 1e-12) and np.allclose(a[:, 61:], 0.0)
    # partially covered boundary pixels carry the exact area fraction
    assert abs(a[7, 30] - 0.5) < 1e-9 and abs(a[30, 5] - 0.75) < 1e-9
    assert abs(a[7, 31] - 0.5 * 255 / 256) < 1e-9


def test_resolved_coverage_is_a_fraction(built):
    fr = oracle.OracleFrame(pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=4, scale=0.01))
    _, cov = fr.masks()
    assert cov.min() >= 0.0 and cov.max() <= 1.0


def test_non_finite_and_huge_segments_end(built):
    """The oracle's tiler ends on a NaN control point (no fills for that
    segment) and on a never-flat cubic (2^20 lines), flagging both."""
    import time
    import oracle
    import pathfinder_gb300 as pf
    for ctrl in ((float("nan"), 10.0), (1e30, -1e30)):
        s = pf.Scene()
        s.set_view_box(pf.RectF(0, 0, 64, 64))
        c = pf.Contour()
        c.push_endpoint(5, 5)
        c.push_cubic(ctrl[0], ctrl[1], -1e30 if ctrl[0] == 1e30 else 30, 40, 50, 50)
        c.push_endpoint(5, 50)
        s.push_draw_path(pf.DrawPath(pf.Outline([c]), pf.ColorU(200, 30, 40, 255)))
        t = time.time()
        fr = oracle.OracleFrame(s)
        assert fr.limit_hit and time.time() - t < 60
