"""Frames in flight on several renderers give exactly the images of one
renderer rendering the same scenes one after another."""
import numpy as np
import pytest

import pathfinder_gb300 as pf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("depth", [2, 3])
def test_pipeline_frames_equal_serial_frames(renderer, depth):
    torch = pytest.importorskip("torch")
    scenes = [pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=s, scale=0.05) for s in (21, 22, 23)]
    scenes.append(pf.generate_scene(pf.PF_SCENE_STARS_512, seed=4))
    scenes.append(pf.generate_scene(pf.PF_SCENE_EDGE_CASES))
    refs = [renderer.render(s) for s in scenes]
    order = [0, 1, 2, 3, 4, 0, 2, 4, 1, 3, 0, 0]
    with pf.RenderPipeline(0, depth=depth) as p:
        outs = [torch.empty((scenes[k].height, scenes[k].width, 4), dtype=torch.uint8).pin_memory().numpy()
                for k in order]
        futs = [p.submit(scenes[k], out) for k, out in zip(order, outs)]
        for k, f in zip(order, futs):
            assert np.array_equal(f.result(), refs[k])
        # forced uploads of one scene, frames into device memory
        dev = [torch.zeros((scenes[0].height, scenes[0].width, 4), dtype=torch.uint8, device="cuda")
               for _ in range(2 * depth)]
        futs = [p.submit(scenes[0], d, force=True) for d in dev]
        for f in futs:
            f.result()
        for d in dev:
            assert np.array_equal(d.cpu().numpy(), refs[0])


def test_image_copy_equals_direct_host_writes(renderer):
    """PF_MEMORY_HOST_COPY (one device-to-host copy after the composite) and
    the composite's own writes into page-locked memory, and pageable memory,
    give the same image; pixels outside the screen tiles keep the buffer's
    contents either way."""
    torch = pytest.importorskip("torch")
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=31, scale=0.05)
    ref = renderer.render(s)
    for pinned in (True, False):
        out = torch.full((s.height, s.width, 4), 7, dtype=torch.uint8)
        out = (out.pin_memory() if pinned else out).numpy()
        renderer.render(s, out=out, copy_image=True)
        assert np.array_equal(out, ref)
    # a target larger than the view box's screen tiles: the margin is kept
    big = torch.full((s.height + 16, s.width + 16, 4), 9, dtype=torch.uint8).pin_memory().numpy()
    direct = big.copy()
    renderer.render(s, out=big, width=s.width + 16, height=s.height + 16, copy_image=True)
    renderer.render(s, out=direct, width=s.width + 16, height=s.height + 16)
    assert np.array_equal(big, direct)
    assert (big[s.height + 8:, :, :] == 9).all()
