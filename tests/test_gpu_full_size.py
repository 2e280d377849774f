"""Full-size parity: the 20,000-path 4K scene the benchmark renders (seed 1,
scale 1.0; also in the D3D11 semantics and with the paint workload) and the
whole 16,384-glyph atlas against the oracle, and scenes
built to reach the composite's long screen-tile lists (33-128 entries, sorted
in shared memory; over 128, sorted in place in global memory), an i8 backdrop
that wraps, and one alpha tile holding hundreds of fills."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from tests.parity import COVERAGE_TOL, compare_images, compare_masks, compare_records

pytestmark = pytest.mark.gpu


def _check_full(renderer, scene, fr):
    """Records bit-exact, raw masks and tile coverage within 1/255 (compared
    tile by tile in the oracle), image within 2/255."""
    img = renderer.render(scene)
    st = renderer.stats()
    assert (st.fill_count, st.tile_count, st.alpha_tile_count) == (fr.fill_count, fr.tile_count,
                                                                   fr.alpha_tile_count)
    compare_records(scene, renderer.read_records(scene), fr)
    ga, gt = renderer.read_masks()
    (ea, et), (wa, wt) = fr.mask_error(ga, gt)
    del ga, gt
    assert ea <= COVERAGE_TOL, f"raw mask error {ea * 255:.3f}/255 in alpha tile {wa}"
    assert et <= COVERAGE_TOL, f"tile coverage error {et * 255:.3f}/255 in path tile {wt}"
    ora, _ = fr.render(scene.width, scene.height)
    compare_images(img, ora)
    return st


def test_svg_4k_full_size_seed1(renderer):
    """The benchmark's frame: 20,000 paths, 2.13M segments, 5.29M fills."""
    import oracle
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=1, scale=1.0)
    fr = oracle.OracleFrame(s)
    assert not fr.limit_hit
    st = _check_full(renderer, s, fr)
    assert st.fill_count > 5_000_000 and st.path_count == 20_000 + len(s.clip_paths)


def test_svg_4k_full_size_d3d11_semantics(built):
    """The same frame in the D3D11 level's tiling semantics (uniform dicing,
    unclipped truncating bins): 3.5M microlines, 5.7M fills."""
    import oracle
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=1, scale=1.0)
    fr = oracle.OracleFrame(s, d3d11=True)
    assert not fr.limit_hit
    with pf.Renderer(0, pf.RendererOptions(d3d11_semantics=True)) as r:
        st = _check_full(r, s, fr)
        assert st.line_count == fr.line_count


def test_svg_4k_full_size_with_paints(renderer):
    """The bench's paint workload at full size (gradients, image patterns with
    filters, blend modes; destructive modes tile the view box, 15M path
    tiles): records bit-exact, and the image against the oracle's FP64
    composite (masks are not read back at this tile count).  The GPU samples
    gradients and blends in FP32 over coverage accumulated in 2^-22 steps,
    and stacks of blend modes with divisions (dodge, burn, the non-separable
    modes' division by the spread of the destination's channels) can amplify
    those differences; so at 33M channel values a few may differ by 3-4/255:
    at most one in a million above 2/255, none above 4/255."""
    import bench
    import oracle
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=1, scale=1.0)
    bench.add_paints(s, 1)
    img = renderer.render(s)
    fr = oracle.OracleFrame(s)
    assert renderer.stats().tile_count == fr.tile_count
    compare_records(s, renderer.read_records(s), fr)
    ora, _ = fr.render(s.width, s.height)
    d = np.abs(img.astype(np.int16) - ora.astype(np.int16))
    assert int((d > 2).sum()) <= d.size // 1_000_000, f"{int((d > 2).sum())} channel values differ by more than 2/255"
    compare_images(img, ora, max_diff=4, frac_exact=0.95)


def test_glyph_atlas_full_size():
    """All 16,384 glyphs: one batched frame equals one frame per glyph byte for
    byte, and every glyph's cell is within 1/255 of the oracle's render of the
    glyph as its own scene."""
    torch = pytest.importorskip("torch")
    import oracle
    atlas = pf.generate_scene(pf.PF_SCENE_GLYPH_ATLAS, seed=1, scale=1.0)
    batch = pf.SceneBatch.glyphs_of(atlas)
    assert len(batch) == 16384
    W, H = atlas.width, atlas.height
    with pf.Renderer(0) as r:
        batched = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
        r.render_batch(batch, batched, pf.PF_CUDA_FORMAT_R8)
        per_glyph = torch.zeros_like(batched)
        for g in range(len(batch)):
            r.render_batch(batch, per_glyph, pf.PF_CUDA_FORMAT_R8, first=g, count=1, sync=False)
        code, _ = r.render_status()
        assert code == 0
        assert torch.equal(batched, per_glyph), "batched atlas differs from per-glyph frames"
        got = batched.cpu().numpy()
    ref = oracle.render_glyphs(atlas)
    d = np.abs(got.astype(np.int16) - ref.astype(np.int16))
    assert d.max() <= 1, f"max diff {d.max()} at {np.argwhere(d > 1)[:4].tolist()}"
    assert (d == 0).mean() >= 0.99


def _scene(w, h):
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, w, h))
    return s


def _rect(x0, y0, x1, y1, reverse=False):
    c = pf.Contour()
    pts = [(x0, y0), (x1, y0), (x1, y1), (x0, y1)]
    if reverse:
        pts = pts[::-1]
    for i, (x, y) in enumerate(pts):
        c.push_endpoint(x, y)
    c.close()
    return c


def _tri(rng, cx, cy, r):
    c = pf.Contour()
    a0 = rng.uniform(0, 2 * np.pi)
    for k in range(3):
        a = a0 + 2 * np.pi * k / 3 + rng.uniform(-0.3, 0.3)
        rr = r * rng.uniform(0.4, 1.0)
        c.push_endpoint(cx + rr * np.cos(a), cy + rr * np.sin(a))
    c.close()
    return c


def _stacked_scene(n, seed):
    """n translucent paths over screen tile (1, 1) of a 64x64 canvas: a third
    cover the tile whole (solid tiles), the rest are triangles and quadratic
    blobs inside or across it (mask tiles), so the tile's visible list has n
    entries in draw order."""
    rng = np.random.default_rng(seed)
    s = _scene(64, 64)
    for i in range(n):
        kind = i % 3
        if kind == 0:
            o = pf.Outline([_rect(12.0 + rng.uniform(0, 3), 13.0 + rng.uniform(0, 2), 35.0 - rng.uniform(0, 2),
                                  34.0 - rng.uniform(0, 3))])
        elif kind == 1:
            o = pf.Outline([_tri(rng, rng.uniform(17, 31), rng.uniform(17, 31), rng.uniform(3, 14))])
        else:
            c = pf.Contour()
            cx, cy, r = rng.uniform(18, 30), rng.uniform(18, 30), rng.uniform(4, 12)
            c.push_endpoint(cx + r, cy)
            for k in range(1, 5):
                a, am = np.pi / 2 * k, np.pi / 2 * (k - 0.5)
                c.push_quadratic(cx + 1.4 * r * np.cos(am), cy + 1.4 * r * np.sin(am),
                                 cx + r * np.cos(a), cy + r * np.sin(a))
            c.close()
            o = pf.Outline([c])
        rule = pf.FillRule.EVEN_ODD if i % 5 == 0 else pf.FillRule.WINDING
        s.push_draw_path(pf.DrawPath(o, pf.ColorU(*[int(v) for v in rng.integers(0, 256, 3)],
                                                  int(rng.integers(20, 200))), rule))
    return s


@pytest.mark.parametrize("n", [40, 100, 200, 300])
def test_long_screen_tile_lists(renderer, n):
    """40 and 100 entries take the shared-memory sort, 200 and 300 the in-place
    sort in global memory."""
    import oracle
    s = _stacked_scene(n, seed=n)
    img = renderer.render(s)
    st = renderer.stats()
    assert st.visible_tile_count >= n
    fr = oracle.OracleFrame(s)
    compare_records(s, renderer.read_records(s), fr)
    compare_masks(renderer, fr)
    ora, _ = fr.render(s.width, s.height)
    compare_images(img, ora)


def test_backdrop_wraps_as_i8(renderer):
    """140 nested squares of one winding in one path: the interior winding
    (140) wraps in the i8 tile backdrop as the reference's does."""
    import oracle
    s = _scene(96, 96)
    contours = [_rect(2.0 + 0.25 * k, 2.0 + 0.25 * k, 94.0 - 0.25 * k, 94.0 - 0.25 * k) for k in range(140)]
    s.push_draw_path(pf.DrawPath(pf.Outline(contours), pf.ColorU(40, 90, 200, 255)))
    img = renderer.render(s)
    fr = oracle.OracleFrame(s)
    rec = renderer.read_records(s)
    compare_records(s, rec, fr)
    assert (rec["tiles"]["backdrop"] < 0).any(), "no tile backdrop wrapped"
    compare_masks(renderer, fr)
    ora, _ = fr.render(s.width, s.height)
    compare_images(img, ora)


def test_hundreds_of_fills_in_one_alpha_tile(renderer):
    """One path of 300 small triangles inside one tile: a single alpha tile
    with hundreds of fills (many accumulation rounds of one mask)."""
    import oracle
    rng = np.random.default_rng(9)
    s = _scene(48, 48)
    s.push_draw_path(pf.DrawPath(pf.Outline([_tri(rng, rng.uniform(18, 30), rng.uniform(18, 30), 2.0)
                                              for _ in range(300)]), pf.ColorU(200, 30, 60, 180),
                                 pf.FillRule.EVEN_ODD))
    img = renderer.render(s)
    st = renderer.stats()
    assert st.fill_count >= 600
    fr = oracle.OracleFrame(s)
    compare_records(s, renderer.read_records(s), fr)
    compare_masks(renderer, fr)
    ora, _ = fr.render(s.width, s.height)
    compare_images(img, ora)
