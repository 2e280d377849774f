"""Stroke to fill on the GPU (PFCUDAStrokeToFill) against the oracle's
restatement of OutlineStrokeToFill: every output point, flag, contour start and
outline start bit-identical; the stroked outlines rendered within the image
bar."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from pathfinder_gb300.stroke import StrokeBatch, outlines_from_buffers
from tests import strokescenes as ss
from tests.parity import compare_images

pytestmark = pytest.mark.gpu


def _both(renderer, items):
    import oracle
    g = renderer.stroke_to_fill_buffers(items)
    batch = StrokeBatch(items)  # the descriptor points into it
    o = oracle.stroke(batch.desc())
    return g, o


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_stroke_bit_exact(renderer, seed):
    (gp, gf, gc, go), (op, of, oc, oo, lim) = _both(renderer, ss.stroke_items(seed))
    assert not lim
    assert np.array_equal(go, oo), "outline starts"
    assert np.array_equal(gc, oc), "contour starts"
    assert gp.shape == op.shape
    bad = np.nonzero(np.any(gp.view(np.uint32) != op.view(np.uint32), axis=1))[0]
    assert len(bad) == 0, f"{len(bad)} points differ, first {bad[:5]}: gpu {gp[bad[:3]]} oracle {op[bad[:3]]}"
    assert np.array_equal(gf, of), "flags"


def test_stroke_then_render(renderer):
    """The stroked outlines drawn as a scene: GPU frame vs oracle frame."""
    import oracle
    items = ss.stroke_items(7, n=30)
    outs = renderer.stroke_to_fill(items)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, 256, 256))
    rng = np.random.default_rng(7)
    for ol in outs:
        s.push_draw_path(pf.DrawPath(ol, pf.ColorU(*[int(v) for v in rng.integers(0, 256, 3)], 200)))
    img = renderer.render(s)
    ora, _ = oracle.OracleFrame(s).render(256, 256)
    compare_images(img, ora)


def test_stroke_device_buffers_and_capacity(renderer):
    """Device-memory input and output, and the capacity status with the sizes needed."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    from pathfinder_gb300 import _abi
    items = ss.stroke_items(11, n=10)
    b = StrokeBatch(items)
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(b, k))).cuda()
           for k in ("points", "flags", "contour_starts", "contour_closed", "outline_starts")}
    styles = torch.frombuffer(bytearray(bytes(b.styles)), dtype=torch.uint8).cuda()
    d = _abi.PFCUDAStrokeInput()
    d.points, d.point_flags = dev["points"].data_ptr(), dev["flags"].data_ptr()
    d.contour_starts, d.contour_closed = dev["contour_starts"].data_ptr(), dev["contour_closed"].data_ptr()
    d.outline_starts, d.styles = dev["outline_starts"].data_ptr(), styles.data_ptr()
    d.point_count, d.contour_count, d.outline_count = len(b.points), b.contour_count, b.outline_count
    d.memory = _abi.PF_MEMORY_DEVICE
    o = _abi.PFCUDAStrokeOutput()
    o.memory = _abi.PF_MEMORY_DEVICE
    rc = renderer._lib.PFCUDAStrokeToFill(renderer._h, C.byref(d), C.byref(o))
    assert rc == _abi.PF_CUDA_ERR_CAPACITY and o.point_count > 0
    n, nc = int(o.point_count), int(o.contour_count)
    pts = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    fl = torch.zeros((n,), dtype=torch.uint8, device="cuda")
    cs = torch.zeros((nc + 1,), dtype=torch.int32, device="cuda")
    os_ = torch.zeros((b.outline_count + 1,), dtype=torch.int32, device="cuda")
    o.points, o.point_flags, o.contour_starts, o.outline_starts = (pts.data_ptr(), fl.data_ptr(), cs.data_ptr(),
                                                                   os_.data_ptr())
    o.point_capacity, o.contour_capacity = n, nc
    assert renderer._lib.PFCUDAStrokeToFill(renderer._h, C.byref(d), C.byref(o)) == 0
    hp, hf, hc, ho = renderer.stroke_to_fill_buffers(items)
    assert np.array_equal(pts.cpu().numpy().view(np.uint32), hp.view(np.uint32))
    assert np.array_equal(fl.cpu().numpy(), hf)
    assert np.array_equal(cs.cpu().numpy().astype(np.uint32), hc)
    assert np.array_equal(os_.cpu().numpy().astype(np.uint32), ho)


def test_stroke_invalid_input(renderer):
    import ctypes as C
    from pathfinder_gb300 import _abi
    items = ss.stroke_items(12, n=3)
    b = StrokeBatch(items)
    b.styles[0].line_cap = 7
    o = _abi.PFCUDAStrokeOutput()
    o.memory = _abi.PF_MEMORY_HOST
    assert renderer._lib.PFCUDAStrokeToFill(renderer._h, C.byref(b.desc()), C.byref(o)) == _abi.PF_CUDA_ERR_INVALID
    b = StrokeBatch(items)
    b.contour_starts[1] = 10 ** 6
    assert renderer._lib.PFCUDAStrokeToFill(renderer._h, C.byref(b.desc()), C.byref(o)) == _abi.PF_CUDA_ERR_INVALID


def test_stroke_huge_input_is_bounded(renderer):
    """A curve that never offsets within tolerance is cut at 2^16 pieces per
    segment: the call ends and reports the limit."""
    from pathfinder_gb300._abi import PFCUDAError
    from pathfinder_gb300.stroke import StrokeStyle
    c = pf.Contour()
    c.push_endpoint(0, 0)
    c.push_cubic(1e30, -1e30, -1e30, 1e30, 50, 50)
    with pytest.raises(PFCUDAError):
        renderer.stroke_to_fill_buffers([(pf.Outline([c]), StrokeStyle(3.0))])
