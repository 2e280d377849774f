"""Edge inputs of the CUDA level against the oracle: a transform, a
background colour, an empty scene, degenerate contours, paths outside or far
outside the view box, one path large enough to overflow every first-frame
capacity, and the async path's capacity status."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from tests.parity import compare_images, compare_masks, compare_records

pytestmark = pytest.mark.gpu


def _check(renderer, scene, options=None):
    import oracle
    img = renderer.render(scene, options=options)
    fr = oracle.OracleFrame(scene, options)
    compare_records(scene, renderer.read_records(scene), fr)
    compare_masks(renderer, fr)
    ora, _ = fr.render(scene.width, scene.height)
    compare_images(img, ora)
    return img


def _star(cx, cy, r0, r1, k, rng=None):
    c = pf.Contour()
    for i in range(2 * k):
        a = np.pi * i / k
        r = r0 if i % 2 == 0 else r1
        x, y = cx + r * np.cos(a), cy + r * np.sin(a)
        if i == 0:
            c.push_endpoint(x, y)
        elif rng is not None and i % 3 == 1:
            c.push_quadratic(x + rng.normal(0, 2), y + rng.normal(0, 2), x, y)
        else:
            c.push_endpoint(x, y)
    c.close()
    return c


def _scene(w, h):
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, w, h))
    return s


def test_transform_parity(renderer):
    s = pf.generate_scene(pf.PF_SCENE_STARS_512, seed=2)
    bo = pf.BuildOptions(pf.Transform2F(0.83, -0.41, 0.37, 0.91, 40.5, -12.25))
    _check(renderer, s, bo)


def test_background_colour(built):
    import oracle
    s = pf.generate_scene(pf.PF_SCENE_STARS_512, seed=3)
    bg = pf.ColorF(0.1, 0.2, 0.3, 0.6)
    with pf.Renderer(0, pf.RendererOptions(background_color=bg)) as r:
        img = r.render(s)
    ora, _ = oracle.OracleFrame(s).render(s.width, s.height, background=(bg.r, bg.g, bg.b, bg.a))
    compare_images(img, ora)


def test_empty_scene(renderer):
    s = _scene(64, 48)
    img = renderer.render(s)
    assert img.shape == (48, 64, 4) and not img.any()
    st = renderer.stats()
    assert st.fill_count == 0 and st.tile_count == 0 and st.visible_tile_count == 0


def test_degenerate_contours(renderer):
    s = _scene(96, 96)
    for pts in ([], [(10, 10)], [(20, 20), (40, 40)], [(30, 30), (30, 30), (30, 30)],
                [(10, 50), (50, 50), (90, 50)]):  # empty, point, segment, repeated, collinear
        c = pf.Contour()
        for p in pts:
            c.push_endpoint(*p)
        if pts:
            c.close()
        s.push_draw_path(pf.DrawPath(pf.Outline([c]), pf.ColorU(200, 10, 10, 255)))
    s.push_draw_path(pf.DrawPath(pf.Outline([_star(48, 48, 30, 12, 7)]), pf.ColorU(10, 200, 10, 180)))
    _check(renderer, s)


def test_paths_outside_and_far_outside_the_view(renderer):
    s = _scene(128, 96)
    rng = np.random.default_rng(4)
    for cx, cy in [(-60, 40), (200, 40), (64, -70), (64, 180), (-50, -50), (190, 150),
                   (64, 48)]:
        s.push_draw_path(pf.DrawPath(pf.Outline([_star(cx, cy, 45, 20, 9, rng)]), pf.ColorU(90, 90, 200, 200)))
    # coordinates far beyond the view on every side, crossing it
    c = pf.Contour()
    for p in [(-1e6, -3e5), (2e6, 40.5), (60.25, 1e6), (-4e5, 70.75)]:
        c.push_endpoint(*p)
    c.close()
    s.push_draw_path(pf.DrawPath(pf.Outline([c]), pf.ColorU(10, 160, 60, 128), pf.FillRule.EVEN_ODD))
    _check(renderer, s)


def test_one_path_beyond_every_first_frame_capacity(built):
    """40,000 edges in one path over 2048^2 (millions of fills): a fresh
    renderer must grow its buffers and re-run the frame (records still
    bit-exact)."""
    rng = np.random.default_rng(5)
    s = _scene(2048, 2048)
    s.push_draw_path(pf.DrawPath(pf.Outline([_star(1024, 1024, 1000, 300, 20_000, rng)]),
                                 pf.ColorU(30, 30, 30, 255)))
    with pf.Renderer(0) as r:
        _check(r, s)


def test_async_capacity_status_then_regrow(built):
    torch = pytest.importorskip("torch")
    from pathfinder_gb300._abi import PF_CUDA_ERR_CAPACITY, PF_CUDA_OK
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=2, scale=0.05)
    out = torch.zeros((s.height, s.width, 4), dtype=torch.uint8, device="cuda")
    with pf.Renderer(0) as r:
        r.upload_scene(s)
        codes = []
        for _ in range(4):  # first-frame capacity guesses may overflow; each status call grows them
            r.render_async(s, out)
            code, _ = r.render_status()
            codes.append(code)
            if code == PF_CUDA_OK:
                break
            assert code == PF_CUDA_ERR_CAPACITY
        assert codes[-1] == PF_CUDA_OK, codes
        ref = r.render(s)
        assert np.array_equal(out.cpu().numpy(), ref)


def test_view_box_away_from_origin_keeps_other_pixels(renderer):
    """Pixels outside the view box's screen tiles keep the buffer's contents,
    for host buffers as for device buffers, whatever the renderer drew before."""
    rng = np.random.default_rng(3)
    big = pf.Scene()
    big.set_view_box(pf.RectF(0, 0, 640, 96))
    big.push_draw_path(pf.DrawPath(pf.Outline([_star(320, 48, 20, 300, 7, rng)]), pf.ColorU(200, 30, 40, 255)))
    renderer.render(big)  # leaves content in the renderer's staging image
    s = pf.Scene()
    s.set_view_box(pf.RectF(500, 8, 640, 96))
    s.push_draw_path(pf.DrawPath(pf.Outline([_star(570, 50, 10, 40, 5, rng)]), pf.ColorU(20, 90, 200, 230)))
    out = np.full((96, 640, 4), 77, np.uint8)
    img = renderer.render(s, out=out)
    x0 = (500 // 16) * 16  # first screen tile column
    assert (img[:, :x0] == 77).all()
    assert (img[40:60, 560:580, 3] > 0).any()


def test_pinned_host_output_matches_pageable(renderer):
    """A page-locked host buffer is written by the composite in place: the
    image equals the pageable render, and pixels outside the screen tiles
    keep the caller's values."""
    import torch
    rng = np.random.default_rng(5)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, 333, 200))
    for _ in range(40):
        s.push_draw_path(pf.DrawPath(pf.Outline([_star(*rng.uniform(0, 333, 2), 5, 60, 7, rng)]),
                                     pf.ColorU(*rng.integers(0, 256, 4).tolist())))
    ref = renderer.render(s, out=np.zeros((200, 333, 4), np.uint8))
    pinned = torch.full((200, 333, 4), 9, dtype=torch.uint8).pin_memory()
    img = renderer.render(s, out=pinned.numpy())
    assert np.array_equal(img, ref)
    # a view box away from the origin: the first tile columns are not drawn
    s.set_view_box(pf.RectF(100, 8, 333, 200))
    pinned.fill_(77)
    img = renderer.render(s, out=pinned.numpy())
    ref = renderer.render(s, out=np.full((200, 333, 4), 77, np.uint8))
    assert np.array_equal(img, ref)
    assert (img[:, :96] == 77).all()
    # an image inside a larger page-locked allocation, rows around it untouched
    big = torch.full((210, 333, 4), 5, dtype=torch.uint8).pin_memory()
    view = big.numpy()[4:204]
    img = renderer.render(s, out=view)
    assert np.array_equal(img[:, 96:], ref[:, 96:]) and (img[:, :96] == 5).all()
    assert (big.numpy()[:4] == 5).all() and (big.numpy()[204:] == 5).all()


def _layout_scene(dx, seed=11):
    rng = np.random.default_rng(seed)
    s = _scene(256, 160)
    for _ in range(30):
        cx, cy = rng.uniform(20, 236), rng.uniform(20, 140)
        s.push_draw_path(pf.DrawPath(pf.Outline([_star(cx + dx, cy, 4, 30, 6, rng)]),
                                     pf.ColorU(*rng.integers(0, 256, 4).tolist())))
    return s


def test_repeated_frames_follow_uploads(renderer):
    """Frames that repeat their layout run as one captured graph from the
    second on: the third frame replays it, and a later upload that keeps every
    size (the same paths moved) shows in the replayed frame."""
    a, b = _layout_scene(0.0), _layout_scene(7.25)
    for _ in range(3):
        _check(renderer, a)
    _check(renderer, b)
    opts = pf.BuildOptions(pf.Transform2F(0.75, 0.1, -0.05, 0.8, 12.5, 3.0))
    for _ in range(3):
        _check(renderer, b, opts)
    _check(renderer, a, opts)


def _bad_point_scene(kind):
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, 64, 64))
    s.push_draw_path(pf.DrawPath(pf.Outline([_star(32, 32, 10, 25, 6)]), pf.ColorU(90, 160, 30, 255)))
    c = pf.Contour()
    c.push_endpoint(5, 5)
    if kind == "nan":
        c.push_cubic(float("nan"), 10, 30, 40, 50, 50)
    else:  # finite but never flat: the walk is bounded per segment
        c.push_cubic(1e30, -1e30, -1e30, 1e30, 50, 50)
    c.push_endpoint(5, 50)
    s.push_draw_path(pf.DrawPath(pf.Outline([c]), pf.ColorU(200, 30, 40, 255)))
    return s


@pytest.mark.parametrize("kind", ["nan", "huge"])
def test_non_finite_and_huge_control_points(renderer, kind):
    """A non-finite segment gives no fills and the frame reports malformed
    input; a finite segment that never flattens is cut at 2^20 lines and the
    frame reports the limit.  Both end promptly, with fills identical to the
    oracle's for the same rules."""
    import oracle
    from pathfinder_gb300._abi import PFCUDAError
    s = _bad_point_scene(kind)
    with pytest.raises(PFCUDAError):
        renderer.render(s)
    fr = oracle.OracleFrame(s)
    assert fr.limit_hit
    compare_records(s, renderer.read_records(s), fr)
