"""Batched frames: many scenes in one set of launches give exactly the pixels
of one frame per scene; graph replay and autotuned launch shapes give exactly
the pixels of a plain frame."""
import numpy as np
import pytest

import pathfinder_gb300 as pf

pytestmark = pytest.mark.gpu


def test_glyph_batch_equals_per_glyph_frames_and_oracle(renderer):
    torch = pytest.importorskip("torch")
    import oracle
    atlas = pf.generate_scene(pf.PF_SCENE_GLYPH_ATLAS, seed=3, scale=0.02)
    batch = pf.SceneBatch.glyphs_of(atlas)
    W, H = atlas.width, atlas.height
    batched = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    renderer.render_batch(batch, batched, pf.PF_CUDA_FORMAT_R8)
    assert renderer.stats().path_count == len(batch)
    per_glyph = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    for g in range(len(batch)):
        renderer.render_batch(batch, per_glyph, pf.PF_CUDA_FORMAT_R8, first=g, count=1, sync=False)
    code, _ = renderer.render_status()
    assert code == 0
    assert torch.equal(batched, per_glyph), "batched atlas differs from per-glyph frames"
    got = batched.cpu().numpy()
    ymax = int(atlas.cells["y1"].max())
    for g in range(0, len(batch), max(1, len(batch) // 24)):
        c = atlas.cells[g]
        img, f64 = oracle.OracleFrame(batch.scenes[g]).render(W, ymax, channels=1)
        cell = (slice(int(c["y0"]), int(c["y1"])), slice(int(c["x0"]), int(c["x1"])))
        d = np.abs(got[cell].astype(int) - img[cell].astype(int))
        assert d.max() <= 1, f"glyph {g}: max diff {d.max()}"


def test_packed_multi_scene_batch_equals_single_frames(renderer):
    torch = pytest.importorskip("torch")
    scenes = [pf.generate_scene(pf.PF_SCENE_STARS_512, seed=s) for s in (1, 2)]
    scenes.append(pf.generate_scene(pf.PF_SCENE_EDGE_CASES))
    scenes.append(pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=9, scale=0.01))
    batch = pf.SceneBatch.packed(scenes)
    out = torch.zeros((batch.total_pixels,), dtype=torch.int32, device="cuda")
    renderer.render_batch(batch, out, pf.PF_CUDA_FORMAT_RGBA8)
    packed = out.cpu().numpy().view(np.uint8)
    for s, off in zip(scenes, batch.offsets):
        single = renderer.render(s)
        part = packed[4 * off:4 * (off + s.width * s.height)].reshape(s.height, s.width, 4)
        assert np.array_equal(part, single)


def test_graph_replay_equals_plain_frame(renderer):
    torch = pytest.importorskip("torch")
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=5, scale=0.02)
    batch = pf.SceneBatch.packed([s])
    ref = torch.zeros((s.height, s.width), dtype=torch.int32, device="cuda")
    renderer.render_batch(batch, ref, pf.PF_CUDA_FORMAT_RGBA8)
    out = torch.zeros_like(ref)
    renderer.graph_capture(batch, out, pf.PF_CUDA_FORMAT_RGBA8)
    out.zero_()
    torch.cuda.synchronize()
    for _ in range(3):
        renderer.graph_launch()
    code, _ = renderer.render_status()
    assert code == 0
    assert torch.equal(out, ref)
    renderer.graph_release()


def test_autotune_changes_speed_not_pixels(renderer):
    torch = pytest.importorskip("torch")
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=6, scale=0.02)
    batch = pf.SceneBatch.packed([s])
    ref = torch.zeros((s.height, s.width), dtype=torch.int32, device="cuda")
    renderer.render_batch(batch, ref, pf.PF_CUDA_FORMAT_RGBA8)
    out = torch.zeros_like(ref)
    best = renderer.autotune(batch, out, pf.PF_CUDA_FORMAT_RGBA8, repeats=2)
    assert best["composite_warps"] in (2, 4, 8) and best["bin_threads"] in (128, 256, 512)
    assert best["composite_batch"] in (1, 2, 4, 8) and best["mask_stage_fills"] in (0, 8, 32)
    for warps, per_item, stage in ((2, 1, 0), (8, 8, 1), (4, 2, 16)):
        renderer.set_tuning(composite_warps=warps, composite_batch=per_item, flatten_threads=64, bin_threads=512,
                            bin_blocks_per_sm=4, mask_stage_fills=stage)
        out.zero_()
        renderer.render_batch(batch, out, pf.PF_CUDA_FORMAT_RGBA8)
        assert torch.equal(out, ref)
    renderer.set_tuning(**best)


@pytest.mark.parametrize("stage", [1, 8, 128])
def test_staged_fill_pass_is_identical(renderer, stage):
    """The fill pass with its fill ranges staged in shared memory by bulk
    copies (the mask_stage_fills knob) writes the same coverage as the
    direct-read default: identical images, paints and clips included."""
    torch = pytest.importorskip("torch")
    from tests import paintscenes
    scenes = [pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=3, scale=0.05), paintscenes.gradient_scene(4),
              paintscenes.pattern_scene(5)]
    default = renderer.get_tuning()
    try:
        for s in scenes:
            ref = renderer.render(s)
            renderer.set_tuning(mask_stage_fills=stage)
            img = renderer.render(s)
            renderer.set_tuning(**default)
            assert np.array_equal(np.asarray(img), np.asarray(ref))
    finally:
        renderer.set_tuning(**default)
    with pytest.raises(pf._abi.PFCUDAError):
        renderer.set_tuning(mask_stage_fills=129)


def test_graph_refused_after_buffers_regrow(built):
    """A captured graph holds the buffers of its capture: once a larger frame
    has regrown them, launching it is refused (it is never replayed on freed
    memory), and a new capture works again."""
    torch = pytest.importorskip("torch")
    from pathfinder_gb300 import _abi
    small = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=12, scale=0.002)
    # 60 translucent full-canvas rectangles: 15 path tiles per screen tile,
    # far above the tile capacity an upload reserves (4 per screen tile)
    big = pf.Scene()
    big.set_view_box(pf.RectF(0, 0, 1024, 1024))
    for k in range(60):
        c = pf.Contour()
        for x, y in ((1.5 + k, 2.5), (1020.5, 1.5 + k), (1019.5 - k, 1021.5), (3.5, 1020.5 - k)):
            c.push_endpoint(x, y)
        c.close()
        big.push_draw_path(pf.DrawPath(pf.Outline([c]), pf.ColorU(k * 4, 255 - k * 4, 90, 40)))
    batch = pf.SceneBatch.packed([small, big])
    out = torch.zeros((batch.total_pixels,), dtype=torch.int32, device="cuda")
    with pf.Renderer(0) as r:
        r.graph_capture(batch, out, pf.PF_CUDA_FORMAT_RGBA8, first=0, count=1)
        r.graph_launch()
        r.render_batch(batch, out, pf.PF_CUDA_FORMAT_RGBA8, first=0, count=2)  # regrows the frame buffers
        with pytest.raises(_abi.PFCUDAError) as e:
            r.graph_launch()
        assert e.value.code == _abi.PF_CUDA_ERR_INVALID
        ref = torch.zeros_like(out)
        r.render_batch(batch, ref, pf.PF_CUDA_FORMAT_RGBA8, first=0, count=1)
        out.zero_()
        r.graph_capture(batch, out, pf.PF_CUDA_FORMAT_RGBA8, first=0, count=1)
        out.zero_()
        r.graph_launch()
        code, _ = r.render_status()
        assert code == 0
        assert torch.equal(out, ref)
