"""The seeded synthetic workloads have the shapes and distributions they are
specified with, and are deterministic."""
import numpy as np

import pathfinder_gb300 as pf


def kinds(scene):
    """Counts of (line, quadratic, cubic) segments as ContourIter yields them."""
    f = scene.flags
    n_line = n_quad = n_cubic = 0
    starts = scene.contour_starts
    for c in range(len(starts) - 1):
        a, b = int(starts[c]), int(starts[c + 1])
        fl = f[a:b]
        i = 0
        n = b - a
        while i < n:
            if i + 1 >= n or fl[i + 1] & 3 == 0:
                n_line += 1; i += 1
            elif fl[i + 2] & 3 == 0:
                n_quad += 1; i += 2
            else:
                n_cubic += 1; i += 3
    return n_line, n_quad, n_cubic


def test_deterministic(built):
    a = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=5, scale=0.05)
    b = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=5, scale=0.05)
    c = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=6, scale=0.05)
    assert np.array_equal(a.points, b.points) and np.array_equal(a.flags, b.flags)
    assert np.array_equal(a.draw_paths, b.draw_paths)
    assert not np.array_equal(a.points[:100], c.points[:100])


def test_svg_4k_distribution(built):
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=1)
    assert (s.width, s.height) == (3840, 2160)
    assert len(s.draw_paths) == 20000
    nseg = s.segment_count
    assert 2.0e6 <= nseg <= 2.25e6
    dp = s.draw_paths
    assert abs((dp["fill_rule"] == 1).mean() - 0.3) < 0.02
    assert abs((dp["paint"][:, 3] < 255).mean() - 0.5) < 0.02
    assert abs((dp["clip_path"] >= 0).mean() - 0.1) < 0.01
    assert len(s.clip_paths) == int((dp["clip_path"] >= 0).sum())
    line, quad, cubic = kinds(pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=1, scale=0.05))
    tot = line + quad + cubic
    # the closing segment of each contour is a line on top of the 40/30/30 edges
    assert abs(quad / tot - 0.3) < 0.03 and abs(cubic / tot - 0.3) < 0.03


def test_stars_512(built):
    s = pf.generate_scene(pf.PF_SCENE_STARS_512, seed=1)
    assert len(s.draw_paths) == 64 and (s.width, s.height) == (512, 512)
    assert s.points.min() >= 0 and s.points.max() <= 512
    assert np.all(s.draw_paths["paint"][:, 3] == 255)
    assert np.all(s.draw_paths["fill_rule"] == 0)
    line, quad, cubic = kinds(s)
    assert quad > 0 and cubic > 0


def test_glyph_atlas_cells(built):
    s = pf.generate_scene(pf.PF_SCENE_GLYPH_ATLAS, seed=1)
    assert len(s.draw_paths) == 16384 and (s.width, s.height) == (4096, 4096)
    cells = s.cells
    occ = np.zeros((4096, 4096), np.uint8)
    for c in cells:
        assert 0 <= c["x0"] < c["x1"] <= 4096 and 0 <= c["y0"] < c["y1"] <= 4096
        occ[c["y0"]:c["y1"], c["x0"]:c["x1"]] += 1
    assert occ.max() == 1, "glyph cells overlap"
    counts = s.draw_paths["contour_count"]
    assert counts.min() >= 1 and counts.max() <= 4
    line, quad, cubic = kinds(pf.generate_scene(pf.PF_SCENE_GLYPH_ATLAS, seed=1, scale=0.02))
    assert cubic == 0 and quad > 0


def test_cubic_1k(built):
    s = pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=1)
    assert len(s.draw_paths) == 256 and len(s.points) == 4096
    line, quad, cubic = kinds(s)
    assert quad == 0 and cubic == 256 * 5
