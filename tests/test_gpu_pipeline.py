"""Frames in flight (PFCUDAPipeline) give exactly the images of one renderer
rendering the same scenes one after another; a frame's error is its own."""
import ctypes as C

import numpy as np
import pytest

import pathfinder_gb300 as pf
from pathfinder_gb300 import _abi

pytestmark = pytest.mark.gpu


def _scenes():
    scenes = [pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=s, scale=0.05) for s in (21, 22, 23)]
    scenes.append(pf.generate_scene(pf.PF_SCENE_STARS_512, seed=4))
    scenes.append(pf.generate_scene(pf.PF_SCENE_EDGE_CASES))
    return scenes


@pytest.mark.parametrize("depth,copy_image", [(1, True), (2, False), (3, True)])
def test_pipeline_frames_equal_serial_frames(renderer, depth, copy_image):
    torch = pytest.importorskip("torch")
    scenes = _scenes()
    refs = [renderer.render(s) for s in scenes]
    order = [0, 1, 2, 3, 4, 0, 2, 4, 1, 3, 0, 0]
    with pf.RenderPipeline(0, depth=depth, copy_image=copy_image) as p:
        outs = [torch.empty((scenes[k].height, scenes[k].width, 4), dtype=torch.uint8).pin_memory().numpy()
                for k in order]
        frames = [p.submit(scenes[k], out) for k, out in zip(order, outs)]
        for k, f in zip(order, frames):
            assert np.array_equal(f.result(), refs[k])
            assert f.done()
        # frames into device memory
        dev = [torch.zeros((scenes[0].height, scenes[0].width, 4), dtype=torch.uint8, device="cuda")
               for _ in range(2 * depth)]
        frames = [p.submit(scenes[0], d) for d in dev]
        for f in frames:
            f.result()
        for d in dev:
            assert np.array_equal(d.cpu().numpy(), refs[0])


def test_pipeline_frame_errors_are_their_own(renderer):
    """A scene the upload refuses fails its frame only; tickets are waited for
    once, and unknown tickets are refused."""
    good = pf.generate_scene(pf.PF_SCENE_STARS_512, seed=5)
    ref = renderer.render(good)
    bad = pf.generate_scene(pf.PF_SCENE_STARS_512, seed=5)
    bad.draw_paths["contour_count"][0] = 1 << 20  # past the scene's contours
    bad.epoch += 1
    with pf.RenderPipeline(0, depth=2) as p:
        outs = [np.zeros((good.height, good.width, 4), np.uint8) for _ in range(4)]
        frames = [p.submit(s, o) for s, o in zip((good, bad, good, bad), outs)]
        for i, f in enumerate(frames):
            if i % 2:
                with pytest.raises(_abi.PFCUDAError) as e:
                    f.result()
                assert e.value.code == _abi.PF_CUDA_ERR_INVALID
            else:
                assert np.array_equal(f.result(), ref)
        L = _abi.lib()
        t = C.c_uint64()
        desc = good.desc()
        out = outs[0]
        assert L.PFCUDAPipelineSubmit(p._h, C.byref(desc), None, good.width, good.height,
                                      C.c_void_p(out.ctypes.data), _abi.PF_MEMORY_HOST, C.byref(t)) == 0
        assert L.PFCUDAPipelineWait(p._h, t.value) == _abi.PF_CUDA_OK
        assert L.PFCUDAPipelineWait(p._h, t.value) == _abi.PF_CUDA_ERR_INVALID
        done = C.c_int32()
        assert L.PFCUDAPipelinePoll(p._h, t.value + 100, C.byref(done)) == _abi.PF_CUDA_ERR_INVALID
        assert np.array_equal(out, ref)


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
    assert (big[s.height:, :, :] == 9).all()


def test_pipeline_frames_of_scenes_with_paints(renderer):
    """A scene with gradients and image patterns gets a new descriptor (and
    new gradient and texel buffers) at every submission: each frame in flight
    keeps its own alive until it is done."""
    torch = pytest.importorskip("torch")
    import bench
    s = pf.generate_scene(pf.PF_SCENE_SVG_4K, seed=41, scale=0.05)
    bench.add_paints(s, 41)
    ref = renderer.render(s)
    with pf.RenderPipeline(0, depth=3) as p:
        outs = [torch.empty((s.height, s.width, 4), dtype=torch.uint8).pin_memory().numpy() for _ in range(9)]
        frames = [p.submit(s, o) for o in outs]
        for f in frames:
            assert np.array_equal(f.result(), ref)
