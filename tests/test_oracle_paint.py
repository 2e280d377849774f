"""Paint effects on the CPU: the reference's gradient tests
(content/src/gradient.rs:278-303) against both the oracle's and the
library's host-side Gradient::sample, ramp equality between the two,
binary16 rounding, and properties of the oracle's blend modes."""
import ctypes as C

import numpy as np
import pytest

import pathfinder_gb300 as pf
from pathfinder_gb300 import _abi
from tests import paintscenes as ps


def _c_gradient(stops_list):
    g = pf.Gradient.linear((0.0, 0.0), (0.0, 0.0))
    g.stops = list(stops_list)  # in the order given: the C side orders them
    return g.to_c()


def _samples(stops_list, ts):
    """(library, oracle) samples at ts."""
    import oracle
    cg, keep = _c_gradient(stops_list)
    L, O = _abi.lib(), oracle.lib()
    lib_out, ora_out = [], []
    for t in ts:
        a, b = _abi.PFColorU(), _abi.PFColorU()
        assert L.PFCUDAGradientSample(C.byref(cg), float(t), C.byref(a)) == 0
        assert O.pfo_gradient_sample(C.byref(cg), C.c_float(t), C.byref(b)) == 0
        lib_out.append((a.r, a.g, a.b, a.a))
        ora_out.append((b.r, b.g, b.b, b.a))
    return lib_out, ora_out


def test_stable_order(built):
    """gradient.rs:278-289: equal offsets keep their insertion order."""
    g = pf.Gradient.linear((0.0, 0.0), (0.0, 0.0))
    for i in range(110):
        g.add_color_stop(pf.ColorU(i, 0, 0, 1), (i % 11) / 10.0)
    st = g.stops
    assert all(a.offset < b.offset or a.color.r < b.color.r for a, b in zip(st, st[1:]))
    # the C side orders stops given out of order the same way
    rng = np.random.default_rng(0)
    shuffled = [pf.ColorStop(pf.ColorU(i, 0, 0, 1), np.float32((i % 11) / 10.0)) for i in range(110)]
    ts = np.linspace(0, 1, 201, dtype=np.float32)
    lib_a, ora_a = _samples(shuffled, ts)
    assert lib_a == ora_a
    lib_b, _ = _samples(st, ts)
    assert lib_a == lib_b, "sorting the insertion order changed the samples"
    del rng


def test_never_sample_zero_width(built):
    """gradient.rs:291-303: a zero-width span is never sampled."""
    stops_list = []
    for i in range(110):
        zero_width = i == 0 or 11 <= i < 99 or i == 109
        stops_list.append(pf.ColorStop(pf.ColorU(255 if zero_width else 0, 0, 0, 1), np.float32((i % 11) / 10.0)))
    ts = [np.float32(i / 10.0) for i in range(11)]
    lib_s, ora_s = _samples(stops_list, ts)
    assert [c[0] for c in lib_s] == [0] * 11
    assert [c[0] for c in ora_s] == [0] * 11


def test_sample_edges(built):
    """No stops: transparent black; t clamped to [0, 1] (NaN to 0)."""
    lib_s, ora_s = _samples([], [0.5])
    assert lib_s == ora_s == [(0, 0, 0, 0)]
    st = [pf.ColorStop(pf.ColorU(10, 20, 30, 40), 0.25), pf.ColorStop(pf.ColorU(200, 100, 0, 255), 0.75)]
    ts = [-1.0, 0.0, 0.25, 0.5, 0.75, 1.0, 7.0, float("nan"), float("inf"), float("-inf")]
    lib_s, ora_s = _samples(st, ts)
    assert lib_s == ora_s
    assert lib_s[0] == (10, 20, 30, 40) and lib_s[6] == (200, 100, 0, 255)
    assert lib_s[7] == lib_s[1]  # NaN clamps to 0


@pytest.mark.parametrize("seed", range(6))
def test_ramp_matches_oracle(built, seed):
    """The library's 256-texel ramp equals the oracle's samples bit for bit."""
    import oracle
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 9))
    offs = rng.uniform(-0.2, 1.2, n).astype(np.float32)
    if seed % 2:
        offs = np.round(offs * 4) / 4  # repeated offsets
    st = [pf.ColorStop(ps.color(rng), float(o)) for o in offs]
    cg, keep = _c_gradient(st)
    ramp = np.zeros((256, 4), np.uint8)
    assert _abi.lib().PFCUDAGradientRamp(C.byref(cg), ramp.ctypes.data) == 0
    O = oracle.lib()
    for x in range(256):
        b = _abi.PFColorU()
        O.pfo_gradient_sample(C.byref(cg), C.c_float((x + 0.5) / 256.0), C.byref(b))
        assert tuple(ramp[x]) == (b.r, b.g, b.b, b.a), x


def test_round_f16_matches_numpy(built):
    """The oracle's binary16 rounding (the metadata texture's f16::from_f32)
    against numpy's float16 conversion."""
    import oracle
    O = oracle.lib()
    rng = np.random.default_rng(3)
    vals = np.concatenate([rng.normal(0, 1, 2000), rng.normal(0, 3000, 2000), rng.uniform(-1e-4, 1e-4, 500),
                           [0.0, -0.0, 65504.0, 65519.0, 65520.0, 1e6, -1e6, 2.0 ** -24, 3 * 2.0 ** -25,
                            2049.0, 2051.0, 4097.0]]).astype(np.float32)
    got = np.array([O.pfo_round_f16(C.c_float(v)) for v in vals], np.float32)
    with np.errstate(over="ignore"):
        want = vals.astype(np.float16).astype(np.float32)
    assert np.array_equal(got, want)


# --- oracle properties of the paint composite --------------------------------
def _render(s, bg=None, channels=4):
    import oracle
    fr = oracle.OracleFrame(s)
    return fr, fr.render(s.width, s.height, background=bg, channels=channels)[1]


def test_constant_gradient_equals_solid(built):
    """A gradient whose stops share one colour paints that colour (SrcIn over
    an opaque white base)."""
    rng = np.random.default_rng(5)
    for kind in ("linear", "radial"):
        s0, s1 = pf.Scene(), pf.Scene()
        for s in (s0, s1):
            s.set_view_box(pf.RectF(0, 0, 64, 64))
        col = pf.ColorU(40, 200, 90, 180)
        out = ps.blob(rng, 32, 32, 24, 10)
        g = ps.linear(rng, 64, 64) if kind == "linear" else ps.radial(rng, 64, 64)
        g.stops = []
        g.add_color_stop(col, 0.2)
        g.add_color_stop(col, 0.9)
        s0.push_draw_path(pf.DrawPath(out, col))
        s1.push_draw_path(pf.DrawPath(out, pf.ColorU(255, 255, 255, 255), gradient=g))
        a, b = _render(s0)[1], _render(s1)[1]
        assert np.abs(a - b).max() < 1e-12


@pytest.mark.parametrize("mode", [pf.BlendMode.CLEAR, pf.BlendMode.COPY, pf.BlendMode.SRC_IN,
                                  pf.BlendMode.MULTIPLY, pf.BlendMode.SCREEN, pf.BlendMode.DIFFERENCE,
                                  pf.BlendMode.LIGHTER, pf.BlendMode.DEST_OUT])
def test_blend_mode_identities(built, mode):
    """Over an opaque backdrop, a path with a known colour: Clear -> 0, Copy ->
    source, SrcIn -> source, Multiply by white, Screen/Difference/Lighter with
    black -> backdrop, DestOut with opaque source -> 0.  Pixels of the path's
    tiles outside the path: Clear, Copy and SrcIn clear them (the blend
    applies over the whole tile quad), the others leave them.  Tiles the path
    does not touch are untouched."""
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, 64, 64))
    s.push_draw_path(pf.DrawPath(ps.rect(-8, -8, 72, 72), pf.ColorU(30, 120, 210, 255)))
    src = {pf.BlendMode.MULTIPLY: pf.ColorU(255, 255, 255, 255), pf.BlendMode.SCREEN: pf.ColorU(0, 0, 0, 255),
           pf.BlendMode.DIFFERENCE: pf.ColorU(0, 0, 0, 255), pf.BlendMode.LIGHTER: pf.ColorU(0, 0, 0, 255)}
    col = src.get(mode, pf.ColorU(200, 50, 10, 255))
    s.push_draw_path(pf.DrawPath(ps.rect(20, 20, 40, 40), col, blend_mode=int(mode)))
    _, img = _render(s)
    back = np.array([30, 120, 210, 255]) / 255.0
    destructive = mode in (pf.BlendMode.CLEAR, pf.BlendMode.COPY, pf.BlendMode.SRC_IN)
    if mode in (pf.BlendMode.CLEAR, pf.BlendMode.DEST_OUT):
        want = np.zeros(4)
    elif mode in (pf.BlendMode.COPY, pf.BlendMode.SRC_IN):
        want = np.array([col.r, col.g, col.b, col.a]) / 255.0
    else:
        want = back
    tol = 1.01 / 255  # the tiler's 8.8 fixed-point fills
    assert np.abs(img[20:40, 20:40] - want).max() < tol
    ring = img[16:20, 16:48]  # in the path's tiles, outside the path
    assert np.abs(ring - (0.0 if destructive else back)).max() < tol
    assert np.abs(img[0:16] - back).max() < 1e-9
    assert np.abs(img[48:] - back).max() < 1e-9


def test_destructive_bounds_and_occlusion(built):
    """Destructive modes tile the whole view box; only opaque paint with
    SrcOver/Clear occludes (renderer/src/builder.rs:80-94, 430-434)."""
    import oracle
    rng = np.random.default_rng(9)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, 96, 80))
    big = ps.rect(2, 2, 94, 78)
    s.push_draw_path(pf.DrawPath(ps.rect(10, 10, 30, 30), pf.ColorU(1, 2, 3, 255), blend_mode=int(pf.BlendMode.COPY)))
    s.push_draw_path(pf.DrawPath(big, pf.ColorU(255, 255, 255, 255), gradient=ps.linear(rng, 96, 80, opaque=True)))
    s.push_draw_path(pf.DrawPath(big, pf.ColorU(255, 255, 255, 255), gradient=ps.linear(rng, 96, 80)))
    s.push_draw_path(pf.DrawPath(big, pf.ColorU(9, 9, 9, 255), blend_mode=int(pf.BlendMode.MULTIPLY)))
    s.push_draw_path(pf.DrawPath(big, pf.ColorU(9, 9, 9, 255), blend_mode=int(pf.BlendMode.CLEAR)))
    fr = oracle.OracleFrame(s)
    _, _, _, rects = fr.tiles()
    assert (rects["x0"][0], rects["y0"][0], rects["x1"][0], rects["y1"][0]) == (0, 0, 6, 5)
    assert (rects["x1"][1] - rects["x0"][1]) == 6
    z = fr.zbuffer().reshape(5, 6)
    # interior tiles: the last occluder is the Clear path (index 4)
    assert (z[1:4, 1:5] == 4).all()
    s.draw_paths["blend_mode"][4] = int(pf.BlendMode.SRC_OVER)
    s.draw_paths["paint"][4] = (9, 9, 9, 200)
    s.epoch += 1
    z = oracle.OracleFrame(s).zbuffer().reshape(5, 6)
    assert (z[1:4, 1:5] == 1).all(), "opaque gradient (index 1) occludes; translucent and Multiply do not"


def test_alpha_only_blend(built):
    """Single-channel renders blend alpha alone: composite modes give 1."""
    s = ps.blend_scene(pf.BlendMode.HUE, seed=2)
    _, a = _render(s, channels=1)
    _, rgba = _render(s)
    assert np.abs(a - rgba[..., 3]).max() < 1e-12


def test_scene_records_paint_fields(built):
    rng = np.random.default_rng(1)
    s = ps.gradient_scene(1)
    assert len(s.gradients) == 7
    g = s.draw_paths["overlay"]
    assert g.max() == 7 and (g[-1] == g[-3])  # the rectangle reuses gradient 6
    s2 = ps.blend_scene(pf.BlendMode.XOR)
    assert (s2.draw_paths["blend_mode"] == int(pf.BlendMode.XOR)).sum() == 2
    d = s.desc()
    assert d.gradient_count == 7 and d.gradients
    del rng


def test_invalid_paint_rejected(built):
    import oracle
    s = ps.blend_scene(pf.BlendMode.SRC_OVER)
    s.draw_paths["blend_mode"][0] = 27
    s.epoch += 1
    with pytest.raises(ValueError):
        oracle.OracleFrame(s)
    s = ps.blend_scene(pf.BlendMode.SRC_OVER)
    s.draw_paths["overlay"][0] = 5  # the scene has no gradients
    s.epoch += 1
    with pytest.raises(ValueError):
        oracle.OracleFrame(s)


# --- image patterns ------------------------------------------------------------
def _pattern_render(pattern, W=48, H=32):
    # view box sides are multiples of the tile size: the CPU tiler clips
    # edges to the view box, so a partial last tile column would stay empty
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    s.push_draw_path(pf.DrawPath(ps.rect(-4, -4, W + 4, H + 4), pf.ColorU(255, 255, 255, 255), pattern=pattern))
    return _render(s)[1]


def test_pattern_placement_nearest(built):
    """Nearest sampling with the identity transform: a non-repeating axis
    has the page's transparent border at pattern coordinate 0 (the image
    starts one texel in, renderer/src/paint.rs:498-530, 617-623); a
    repeating axis tiles the image from 0."""
    rng = np.random.default_rng(1)
    img = ps.image(rng, 7, 5, opaque=True)
    for rx, ry in ((False, False), (True, True), (True, False)):
        p = pf.Pattern.from_image(img)
        p.repeat_x, p.repeat_y, p.smoothing = rx, ry, False
        out = _pattern_render(p)
        for y in range(32):
            for x in range(48):
                ix = x % 7 if rx else x - 1
                iy = y % 5 if ry else y - 1
                want = img[iy, ix] / 255.0 if (0 <= ix < 7 and 0 <= iy < 5) else np.zeros(4)
                want = np.concatenate([want[:3] * want[3], want[3:]])
                assert np.abs(out[y, x] - want).max() < 1e-9, (rx, ry, x, y)


def test_pattern_filters(built):
    """A colour matrix swapping red and blue; a blur of a constant image."""
    rng = np.random.default_rng(2)
    img = ps.image(rng, 6, 6, opaque=True)
    p = pf.Pattern.from_image(img)
    p.repeat_x = p.repeat_y = True
    p.smoothing = False
    cols = np.zeros((5, 4), np.float32)
    cols[0] = (0, 0, 1, 0)
    cols[1] = (0, 1, 0, 0)
    cols[2] = (1, 0, 0, 0)
    cols[3] = (0, 0, 0, 1)
    plain = _pattern_render(p)
    p.set_color_matrix(cols)
    swapped = _pattern_render(p)
    assert np.abs(swapped[..., [2, 1, 0, 3]] - plain).max() < 1e-9
    flat = np.zeros((8, 8, 4), np.uint8)
    flat[...] = (40, 120, 200, 255)
    q = pf.Pattern.from_image(flat)
    q.repeat_x = q.repeat_y = True
    for sigma, d in ((0.7, "x"), (2.5, "y"), (9.0, "x")):
        q.set_blur(sigma, d)
        out = _pattern_render(q)
        assert np.abs(out - np.array([40, 120, 200, 255]) / 255.0).max() < 1e-6, sigma


def test_pattern_occlusion_follows_image_opacity(built):
    """Image::is_opaque decides occlusion (content/src/pattern.rs:193-195,
    208-212), also for a non-repeating pattern whose page border is
    transparent: the tiles it covers hide what lies below."""
    import oracle
    rng = np.random.default_rng(3)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, 64, 64))
    s.push_draw_path(pf.DrawPath(ps.rect(0, 0, 64, 64), pf.ColorU(10, 200, 30, 255)))
    p = pf.Pattern.from_image(ps.image(rng, 4, 4, opaque=True))
    s.push_draw_path(pf.DrawPath(ps.rect(-8, -8, 72, 72), pf.ColorU(255, 255, 255, 255), pattern=p))
    z = oracle.OracleFrame(s).zbuffer()
    assert (z == 1).all()
    img = _render(s)[1]
    assert np.abs(img[40:, 40:]).max() == 0  # transparent: the green below is culled
