"""Dashes on the GPU (PFCUDADashOutlines, PFCUDAStrokeToFillDashed) against the
oracle's restatement of OutlineDash (content/src/dash.rs:18-152): every output
point, flag, contour start, closed flag and outline start bit-identical, and a
dashed stroke identical to the oracle's dash followed by its stroke."""
import ctypes as C

import numpy as np
import pytest

import pathfinder_gb300 as pf
from pathfinder_gb300 import _abi
from pathfinder_gb300.stroke import LineCap, LineJoin, StrokeBatch, StrokeStyle
from tests import strokescenes as ss

pytestmark = pytest.mark.gpu


def dash_items(seed, n=40, negative=True):
    """The seeded stroke outlines with seeded patterns: even and odd lengths,
    zero-length dashes, negative (unless not `negative`), zero and large
    offsets, some outlines without a pattern."""
    rng = np.random.default_rng(1000 + seed)
    items = []
    for ol, st in ss.stroke_items(seed, n=n):
        kind = int(rng.integers(0, 6))
        if kind == 0:
            dashes = []
        elif kind == 1:
            dashes = [0.0, float(rng.uniform(2, 9))]
        else:
            dashes = [float(x) for x in rng.uniform(0.5, 25.0, int(rng.integers(1, 6)))]
        offset = float(rng.choice([0.0, rng.uniform(-40 if negative else 0, 40), rng.uniform(0, 500), 3.0]))
        items.append((ol, st, dashes, offset))
    return items


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _differ(a, b):
    """Points whose coordinates differ in bits, a NaN matching any NaN: a
    negative offset over a zero-length segment cuts it at t = -inf, which
    gives NaN as in the reference (0 * inf), and x86 and the GPU write
    different NaN bits."""
    same = (_bits(a) == _bits(b)) | (np.isnan(a) & np.isnan(b))
    return np.nonzero(~np.all(same, axis=1))[0]


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_dash_bit_exact(renderer, seed):
    import oracle
    items = dash_items(seed)
    gp, gf, gc, gcl, go = renderer.dash_buffers([(ol, d, off) for ol, _, d, off in items])
    b = StrokeBatch(items)
    op, of, oc, ocl, oo, lim = oracle.dash(b.desc(), b.dash_desc())
    assert not lim
    assert np.array_equal(go, oo), "outline starts"
    assert np.array_equal(gc, oc), "contour starts"
    assert np.array_equal(gcl, ocl), "closed flags"
    assert gp.shape == op.shape
    bad = _differ(gp, op)
    assert len(bad) == 0, f"{len(bad)} points differ, first {bad[:5]}: gpu {gp[bad[:3]]} oracle {op[bad[:3]]}"
    assert np.array_equal(gf, of), "flags"


@pytest.mark.parametrize("seed", [0, 4])
def test_dashed_stroke_is_dash_then_stroke(renderer, seed):
    """PFCUDAStrokeToFillDashed against the oracle's dash fed to its stroke,
    with every cap and join (offsets from 0 up: a negative offset over a
    zero-length segment gives NaN points, which the stroker cannot offset)."""
    import oracle
    items = dash_items(seed, n=30, negative=False)
    gp, gf, gc, go = renderer.stroke_to_fill_buffers(items)
    b = StrokeBatch(items)
    dp, df, dc, dcl, do, _ = oracle.dash(b.desc(), b.dash_desc())
    sin = _abi.PFCUDAStrokeInput()
    dp = np.ascontiguousarray(dp)
    sin.points, sin.point_flags = dp.ctypes.data, df.ctypes.data
    dcl1 = dcl if len(dcl) else np.zeros((1,), np.uint8)
    sin.contour_starts, sin.contour_closed, sin.outline_starts = dc.ctypes.data, dcl1.ctypes.data, do.ctypes.data
    sin.styles = C.addressof(b.styles)
    sin.point_count, sin.contour_count, sin.outline_count = len(dp), len(dcl), b.outline_count
    sin.memory = _abi.PF_MEMORY_HOST
    op, of, oc, oo, lim = oracle.stroke(sin)
    assert not lim
    assert np.array_equal(go, oo) and np.array_equal(gc, oc)
    assert gp.shape == op.shape
    assert len(_differ(gp, op)) == 0, "points"
    assert np.array_equal(gf, of), "flags"


def test_dashed_stroke_renders(renderer):
    """Round-capped dots and dashes drawn as a scene: the GPU frame against the
    oracle's frame within the image bar."""
    import oracle
    from tests.parity import compare_images
    c = pf.Contour().push_endpoint(10, 20).push_endpoint(200, 40)
    c.push_cubic(240, 80, 120, 200, 40, 230)
    items = [(pf.Outline([c]), StrokeStyle(6.0, LineCap.ROUND, LineJoin.ROUND), [0.0, 14.0], 0.0),
             (pf.Outline([c]), StrokeStyle(2.0, LineCap.BUTT, LineJoin.MITER), [9.0, 4.0, 2.0, 4.0], 5.0)]
    outs = renderer.stroke_to_fill(items)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, 256, 256))
    for ol, color in zip(outs, [pf.ColorU(200, 30, 30, 255), pf.ColorU(20, 40, 220, 200)]):
        s.push_draw_path(pf.DrawPath(ol, color))
    img = renderer.render(s)
    ora, _ = oracle.OracleFrame(s).render(256, 256)
    compare_images(img, ora)
    assert (np.asarray(img)[..., 3] > 0).sum() > 500


def test_dash_device_memory(renderer):
    """Input and output in device memory give the host-memory result."""
    torch = pytest.importorskip("torch")
    items = dash_items(5, n=12)
    hp, hf, hc, hcl, ho = renderer.dash_buffers([(ol, d, off) for ol, _, d, off in items])
    b = StrokeBatch(items)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tp, tf, tc, tcl, to = dev(b.points), dev(b.flags), dev(b.contour_starts), dev(b.contour_closed), dev(b.outline_starts)
    td, tds, tdo = dev(b.dashes), dev(b.dash_starts), dev(b.dash_offsets)
    sin = b.desc()
    sin.points, sin.point_flags, sin.contour_starts = tp.data_ptr(), tf.data_ptr(), tc.data_ptr()
    sin.contour_closed, sin.outline_starts, sin.memory = tcl.data_ptr(), to.data_ptr(), _abi.PF_MEMORY_DEVICE
    dd = _abi.PFCUDADashInput(td.data_ptr(), tds.data_ptr(), tdo.data_ptr())
    P, NC = len(hp), len(hcl)
    op = torch.zeros((P, 2), dtype=torch.float32, device="cuda")
    of = torch.zeros((P,), dtype=torch.uint8, device="cuda")
    oc = torch.zeros((NC + 1,), dtype=torch.int32, device="cuda")
    ocl = torch.zeros((max(NC, 1),), dtype=torch.uint8, device="cuda")
    oo = torch.zeros((b.outline_count + 1,), dtype=torch.int32, device="cuda")
    out = _abi.PFCUDAOutlineOutput(op.data_ptr(), of.data_ptr(), oc.data_ptr(), ocl.data_ptr(), oo.data_ptr(),
                                   P, NC, 0, 0, _abi.PF_MEMORY_DEVICE)
    L = _abi.lib()
    assert L.PFCUDADashOutlines(renderer._h, C.byref(sin), C.byref(dd), C.byref(out)) == _abi.PF_CUDA_OK
    assert out.point_count == P and out.contour_count == NC
    assert np.array_equal(op.cpu().numpy().view(np.uint32), hp.view(np.uint32))
    assert np.array_equal(of.cpu().numpy(), hf)
    assert np.array_equal(oc.cpu().numpy().astype(np.uint32), hc)
    assert np.array_equal(ocl.cpu().numpy()[:NC], hcl)
    assert np.array_equal(oo.cpu().numpy().astype(np.uint32), ho)


def test_dash_rejects_bad_patterns(renderer):
    ol = pf.Outline([pf.Contour().push_endpoint(0, 0).push_endpoint(8, 0)])
    for dashes, offset in [([-1.0, 2.0], 0.0), ([0.0, 0.0], 0.0), ([1.0, float("nan")], 0.0),
                           ([1.0, 2.0], float("inf")), ([float("inf"), 1.0], 0.0)]:
        with pytest.raises(_abi.PFCUDAError) as e:
            renderer.dash_buffers([(ol, dashes, offset)])
        assert e.value.code == _abi.PF_CUDA_ERR_INVALID


def test_dash_capacity_and_counts(renderer):
    """Too little capacity: PF_CUDA_ERR_CAPACITY with the sizes needed."""
    items = dash_items(6, n=8)
    b = StrokeBatch(items)
    out = _abi.PFCUDAOutlineOutput()
    pts = np.zeros((1, 2), np.float32)
    fl = np.zeros((1,), np.uint8)
    cs = np.zeros((2,), np.uint32)
    cl = np.zeros((1,), np.uint8)
    os_ = np.zeros((b.outline_count + 1,), np.uint32)
    out.points, out.point_flags, out.contour_starts = pts.ctypes.data, fl.ctypes.data, cs.ctypes.data
    out.contour_closed, out.outline_starts = cl.ctypes.data, os_.ctypes.data
    out.point_capacity, out.contour_capacity, out.memory = 1, 1, _abi.PF_MEMORY_HOST
    rc = _abi.lib().PFCUDADashOutlines(renderer._h, C.byref(b.desc()), C.byref(b.dash_desc()), C.byref(out))
    assert rc == _abi.PF_CUDA_ERR_CAPACITY
    hp, _, _, hcl, _ = renderer.dash_buffers([(ol, d, off) for ol, _, d, off in items])
    assert out.point_count == len(hp) and out.contour_count == len(hcl)


def test_dash_step_bound(renderer):
    """A pattern too fine for its outline stops after 2^20 steps: the call
    returns PF_CUDA_ERR_LIMIT and its output up to there equals the oracle's
    (which stops at the same step)."""
    import oracle
    ol = pf.Outline([pf.Contour().push_endpoint(0, 0).push_endpoint(3000, 0)])
    items = [(ol, None, [0.001, 0.001], 0.0)]
    b = StrokeBatch(items)
    op, of, oc, ocl, oo, lim = oracle.dash(b.desc(), b.dash_desc())
    assert lim
    P, NC = len(op), len(ocl)
    pts = np.zeros((P, 2), np.float32)
    fl = np.zeros((P,), np.uint8)
    cs = np.zeros((NC + 1,), np.uint32)
    cl = np.zeros((NC,), np.uint8)
    os_ = np.zeros((2,), np.uint32)
    out = _abi.PFCUDAOutlineOutput(pts.ctypes.data, fl.ctypes.data, cs.ctypes.data, cl.ctypes.data, os_.ctypes.data,
                                   P, NC, 0, 0, _abi.PF_MEMORY_HOST)
    rc = _abi.lib().PFCUDADashOutlines(renderer._h, C.byref(b.desc()), C.byref(b.dash_desc()), C.byref(out))
    assert rc == _abi.PF_CUDA_ERR_LIMIT
    assert out.point_count == P and out.contour_count == NC
    assert np.array_equal(pts.view(np.uint32), op.view(np.uint32))
    assert np.array_equal(cs, oc) and np.array_equal(os_, oo)
