"""Paint effects on the GPU: every blend mode, every gradient kind and wrap,
image patterns with their filters,
gradients under a build transform, in batches and in the alpha-only format.
Records bit-exact with the oracle (destructive modes tile the view box,
occlusion follows the paint's opacity and blend mode), images within 2/255
of the oracle's FP64 composite."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from tests import paintscenes as ps
from tests.parity import compare_images, compare_records

pytestmark = pytest.mark.gpu


def _check(renderer, s, options=None, frac_exact=0.97, bg=None):
    import oracle
    img = renderer.render(s, options)
    fr = oracle.OracleFrame(s, options)
    compare_records(s, renderer.read_records(s), fr)
    ora, _ = fr.render(s.width, s.height, background=bg)
    try:
        return compare_images(img, ora, frac_exact=frac_exact)
    except AssertionError as e:
        raise AssertionError(f"{e}; tuning {renderer.get_tuning()}") from None


@pytest.mark.parametrize("mode", list(pf.BlendMode))
def test_blend_mode_parity(renderer, mode):
    _check(renderer, ps.blend_scene(mode, seed=1, gradient=True))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_gradient_parity(renderer, seed):
    _check(renderer, ps.gradient_scene(seed))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_pattern_parity(renderer, seed):
    """Image patterns: every repeat/smoothing combination, rotated and
    scaled, blur and colour-matrix filters."""
    _check(renderer, ps.pattern_scene(seed))


def test_pattern_under_transform(renderer):
    s = ps.pattern_scene(5, W=256, H=192)
    t = pf.Transform2F(0.9, 0.35, -0.3, 1.1, 12.5, -7.0)
    _check(renderer, s, pf.BuildOptions(t))


def test_gradient_under_transform(renderer):
    """The colour texture transform composes the inverse build transform and is
    rounded to binary16: a rotation, scale and offset that make the rounding
    visible at these coordinates."""
    s = ps.gradient_scene(4, W=320, H=256, clip=False)
    c, sn = np.cos(0.3), np.sin(0.3)
    t = pf.Transform2F(1.3 * c, -1.3 * sn, 1.3 * sn, 1.3 * c, 37.25, -12.5)
    _check(renderer, s, pf.BuildOptions(t))


def test_large_coordinates(renderer):
    """Gradients far from the origin (binary16 spacing of 2-4 px there)."""
    rng = np.random.default_rng(7)
    s = pf.Scene()
    W, H = 3000, 160
    s.set_view_box(pf.RectF(2600, 0, W, H))
    for k in range(3):
        g = pf.Gradient.linear((2620 + 90 * k, 10), (2900 - 40 * k, 150))
        ps.stops(g, rng)
        r = pf.Gradient.radial((2700 + 100 * k, 80.0), (5.0, 120.0))
        ps.stops(r, rng)
        s.push_draw_path(pf.DrawPath(ps.blob(rng, 2700 + 120 * k, 80, 70, 10), pf.ColorU(255, 255, 255, 220),
                                     gradient=g if k % 2 else r))
    _check(renderer, s)


def test_background_and_destructive(renderer):
    """Destructive modes over a background colour: cleared pixels take the
    mode's result, not the background."""
    bg = pf.ColorF(0.2, 0.4, 0.6, 0.8)
    import oracle
    with pf.Renderer(0, pf.RendererOptions(background_color=bg)) as r:
        for mode in (pf.BlendMode.CLEAR, pf.BlendMode.SRC_IN, pf.BlendMode.DEST_ATOP, pf.BlendMode.COLOR_DODGE):
            s = ps.blend_scene(mode, seed=3)
            img = r.render(s)
            fr = oracle.OracleFrame(s)
            ora, _ = fr.render(s.width, s.height, background=(bg.r, bg.g, bg.b, bg.a))
            compare_images(img, ora, frac_exact=0.97)


def test_alpha_only_format(renderer):
    """R8 output blends alpha alone (composite modes give 1)."""
    import oracle
    torch = pytest.importorskip("torch")
    for mode in (pf.BlendMode.SRC_OVER, pf.BlendMode.XOR, pf.BlendMode.DEST_IN, pf.BlendMode.SCREEN):
        s = ps.blend_scene(mode, seed=5, gradient=True)
        batch = pf.SceneBatch.packed([s])
        out = torch.zeros((s.height, s.width), dtype=torch.uint8, device="cuda")
        renderer.render_batch(batch, out, pf.PF_CUDA_FORMAT_R8)
        ora, _ = oracle.OracleFrame(s).render(s.width, s.height, channels=1)
        compare_images(out.cpu().numpy(), ora, frac_exact=0.97)


def test_batch_with_gradients(renderer):
    """Scenes of one batch keep their own gradients and blend modes."""
    import oracle
    torch = pytest.importorskip("torch")
    scenes = [ps.gradient_scene(10 + k, W=96 + 16 * k, H=80) for k in range(3)]
    scenes.insert(1, ps.blend_scene(pf.BlendMode.MULTIPLY, seed=2, gradient=True))
    batch = pf.SceneBatch.packed(scenes)
    out = torch.zeros((batch.total_pixels,), dtype=torch.int32, device="cuda")
    renderer.render_batch(batch, out, pf.PF_CUDA_FORMAT_RGBA8)
    packed = out.cpu().numpy().view(np.uint8)
    for s, off in zip(scenes, batch.offsets):
        img = packed[4 * off:4 * (off + s.width * s.height)].reshape(s.height, s.width, 4)
        ora, _ = oracle.OracleFrame(s).render(s.width, s.height)
        compare_images(img, ora, frac_exact=0.97)


def test_invalid_paint_rejected(renderer):
    from pathfinder_gb300._abi import PFCUDAError
    s = ps.blend_scene(pf.BlendMode.SRC_OVER)
    s.draw_paths["blend_mode"][1] = 27
    s.epoch += 1
    with pytest.raises(PFCUDAError):
        renderer.render(s)
    s = ps.gradient_scene(0)
    s.draw_paths["overlay"][-1] = 99
    s.epoch += 1
    with pytest.raises(PFCUDAError):
        renderer.render(s)


def test_differentiable_frame_rejects_paint_effects(renderer):
    """The adjoint covers solid SrcOver paint: other paint is refused."""
    from pathfinder_gb300._abi import PFCUDAError
    torch = pytest.importorskip("torch")
    s = ps.blend_scene(pf.BlendMode.MULTIPLY)
    renderer.upload_scene(s, force=True)
    out = torch.zeros((s.height, s.width), dtype=torch.float32, device="cuda")
    with pytest.raises(PFCUDAError):
        renderer.render_diff(out, width=s.width, height=s.height)


def test_svg4k_with_paints_reduced(renderer):
    """The bench's paint workload (gradients on a quarter of the paths, blend
    modes on a tenth) at a tenth of the 4K scene's paths."""
    import bench
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=3, scale=0.1)
    bench.add_paints(s, 3)
    _check(renderer, s, frac_exact=0.95)
