"""Scene upload through the C ABI. The per-path tables, the contour order and
the clip-chain checks are built on the device: every invalid record is
refused (fill rule, blend mode, contour range, clip index, a clip path
clipping itself, overlay index, contour boundaries), a refused upload leaves
the renderer usable, contour boundaries may sit in device memory, and paths
may share contours (more references than contours)."""
import ctypes as C

import numpy as np
import pytest

import pathfinder_gb300 as pf
from pathfinder_gb300 import _abi
from tests.parity import compare_images

pytestmark = pytest.mark.gpu


def _star(cx, cy, r0, r1, k):
    c = pf.Contour()
    for i in range(2 * k):
        a = np.pi * i / k
        r = r0 if i % 2 == 0 else r1
        x, y = cx + r * np.cos(a), cy + r * np.sin(a)
        if i % 4 == 1:
            c.push_quadratic(x + 3.0, y - 2.0, x, y)
        else:
            c.push_endpoint(x, y)
    c.close()
    return c


def _scene(seed=3):
    rng = np.random.default_rng(seed)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, 240, 160))
    c0 = s.push_clip_path(pf.ClipPath(pf.Outline([_star(120, 80, 70, 40, 9)])))
    for _ in range(12):
        cx, cy = rng.uniform(20, 220), rng.uniform(20, 140)
        s.push_draw_path(pf.DrawPath(pf.Outline([_star(cx, cy, 8, 35, 6), _star(cx + 9, cy, 4, 12, 5)]),
                                     pf.ColorU(*rng.integers(0, 256, 4).tolist()),
                                     clip_path=c0 if rng.uniform() < 0.5 else None))
    return s


def _render(renderer, s):
    return renderer.render(s, out=np.zeros((s.height, s.width, 4), np.uint8))


def _mutations():
    def rule(s): s.draw_paths["fill_rule"][3] = 2
    def blend(s): s.draw_paths["blend_mode"][2] = 99
    def contour_range(s): s.draw_paths["contour_count"][5] = len(s.contour_starts)
    def clip_index(s): s.draw_paths["clip_path"][1] = 1
    def self_clip(s): s.clip_paths["clip_path"][0] = 0
    def overlay(s): s.draw_paths["overlay"][4] = 1
    def starts_order(s): s.contour_starts[6], s.contour_starts[7] = s.contour_starts[7], s.contour_starts[6]
    def starts_past_points(s): s.contour_starts[-1] = len(s.points) + 1
    return [rule, blend, contour_range, clip_index, self_clip, overlay, starts_order, starts_past_points]


@pytest.mark.parametrize("mutate", _mutations(), ids=lambda f: f.__name__)
def test_invalid_records_refused_then_valid_upload(renderer, mutate):
    good = _scene()
    ref = _render(renderer, good)
    bad = _scene()
    mutate(bad)
    bad.epoch += 1
    with pytest.raises(_abi.PFCUDAError):
        renderer.upload_scene(bad, force=True)
    out = np.zeros((good.height, good.width, 4), np.uint8)
    code = renderer._lib.PFCUDARenderScene(renderer._h, C.byref(pf.BuildOptions().to_c()), good.width, good.height,
                                           C.c_void_p(out.ctypes.data), _abi.PF_MEMORY_HOST)
    assert code == _abi.PF_CUDA_ERR_NO_SCENE  # no scene after a refused upload
    renderer.upload_scene(good, force=True)
    assert np.array_equal(_render(renderer, good), ref)


def test_contour_boundaries_in_device_memory(renderer):
    torch = pytest.importorskip("torch")
    s = _scene(5)
    ref = _render(renderer, s)
    pts = torch.from_numpy(s.points.copy()).cuda()
    flags = torch.from_numpy(s.flags.copy()).cuda()
    starts = torch.from_numpy(s.contour_starts.astype(np.uint32).copy()).cuda()
    d = s.desc()
    d.points, d.point_flags, d.contour_starts = pts.data_ptr(), flags.data_ptr(), starts.data_ptr()
    d.memory = _abi.PF_MEMORY_DEVICE
    _abi.check(renderer._lib.PFCUDASceneUpload(renderer._h, C.byref(d)), "PFCUDASceneUpload")
    out = np.zeros_like(ref)
    _abi.check(renderer._lib.PFCUDARenderScene(renderer._h, C.byref(pf.BuildOptions().to_c()), s.width, s.height,
                                               C.c_void_p(out.ctypes.data), _abi.PF_MEMORY_HOST), "render")
    assert np.array_equal(out, ref)


def test_paths_sharing_contours(renderer):
    """Every draw path drawing all the draw paths' contours: 12 x 24
    references of 26 contour slots, so the order buffers grow after packing.
    The image equals a scene that repeats the outline in each path."""
    import oracle
    s = _scene(7)
    first = int(s.draw_paths["first_contour"][0])
    count = int(s.draw_paths["contour_count"].sum())
    assert first + count == len(s.contour_starts) - 1
    s.draw_paths["first_contour"][:] = first
    s.draw_paths["contour_count"][:] = count
    s.epoch += 1
    img = _render(renderer, s)

    def contour(c):
        p0, p1 = int(s.contour_starts[c]), int(s.contour_starts[c + 1])
        k = pf.Contour()
        k.points = [(float(x), float(y)) for x, y in s.points[p0:p1]]
        k.flags = [int(f) for f in s.flags[p0:p1]]
        k.closed = True
        return k

    t = pf.Scene()
    t.set_view_box(s.view_box)
    t.push_clip_path(pf.ClipPath(pf.Outline([_star(120, 80, 70, 40, 9)])))
    for i in range(len(s.draw_paths)):
        dp = s.draw_paths[i]
        outline = pf.Outline([contour(c) for c in range(first, first + count)])
        t.push_draw_path(pf.DrawPath(outline, pf.ColorU(*[int(v) for v in dp["paint"]]),
                                     clip_path=0 if dp["clip_path"] >= 0 else None))
    ref = _render(renderer, t)
    assert np.array_equal(img, ref)
    ora, _ = oracle.OracleFrame(t).render(t.width, t.height)
    compare_images(img, ora)
