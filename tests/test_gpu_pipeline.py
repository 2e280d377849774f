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
