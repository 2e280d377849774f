"""The CUDA renderer level behind the reference's Renderer API shape
(renderer/src/gpu/renderer.rs:76-460, renderer/src/gpu/options.rs:19-46,
renderer/src/options.rs:53-61), over the C ABI in include/pathfinder_cuda.h.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from enum import IntEnum

import numpy as np

from . import _abi
from .scene import ColorF, Scene

_FILL, _TILE, _CLIP, _PATH, _RECT = _abi.record_dtypes()


class RendererLevel(IntEnum):
    """renderer/src/gpu/options.rs:41-46, extended with the CUDA level."""
    D3D9 = 0
    D3D11 = 1
    CUDA = 2


@dataclass
class Transform2F:
    """Row-major 2x3 affine transform (geometry/src/transform2d.rs:187-192)."""
    m00: float = 1.0
    m01: float = 0.0
    m10: float = 0.0
    m11: float = 1.0
    tx: float = 0.0
    ty: float = 0.0


@dataclass
class BuildOptions:
    """renderer/src/options.rs:53-61 (transform only on this path)."""
    transform: Transform2F | None = None

    def to_c(self) -> _abi.PFCUDABuildOptions:
        o = _abi.PFCUDABuildOptions()
        if self.transform is not None:
            t = self.transform
            o.transform = _abi.PFTransform2F(t.m00, t.m01, t.m10, t.m11, _abi.PFVector2F(t.tx, t.ty))
            o.has_transform = 1
        return o


@dataclass
class RendererOptions:
    """renderer/src/gpu/options.rs:19-33.  d3d11_semantics tiles as the D3D11
    level does (uniform dicing, unclipped truncating bins) instead of as the
    CPU tiler does (PF_CUDA_RENDERER_D3D11_SEMANTICS)."""
    background_color: ColorF | None = None
    d3d11_semantics: bool = False

    def to_c(self) -> _abi.PFCUDARendererOptions:
        o = _abi.PFCUDARendererOptions()
        if self.background_color is not None:
            c = self.background_color
            o.background_color = _abi.PFColorF(c.r, c.g, c.b, c.a)
            o.has_background_color = 1
        if self.d3d11_semantics:
            o.flags |= _abi.PF_CUDA_RENDERER_D3D11_SEMANTICS
        return o


@dataclass
class RenderStats:
    """renderer/src/gpu/perf.rs:21-44 plus the device counters of the frame."""
    path_count: int = 0
    segment_count: int = 0
    line_count: int = 0
    fill_count: int = 0
    tile_count: int = 0
    alpha_tile_count: int = 0
    visible_tile_count: int = 0
    screen_tile_count: int = 0
    status: int = 0
    gpu_time_ms: float = 0.0
    kernel_launches: int = 0
    mask_tile_count: int = 0
    mask_fill_count: int = 0


def _ptr(x):
    """(address, memory kind) of a numpy array or a torch tensor."""
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("output array must be C-contiguous")
        return x.ctypes.data, _abi.PF_MEMORY_HOST
    try:
        import torch
        if isinstance(x, torch.Tensor):
            if not x.is_contiguous():
                raise ValueError("output tensor must be contiguous")
            return x.data_ptr(), (_abi.PF_MEMORY_DEVICE if x.is_cuda else _abi.PF_MEMORY_HOST)
    except ImportError:
        pass
    raise TypeError(f"unsupported output buffer {type(x)}")


class Renderer:
    """Renderer::new / render_command / end_scene for RendererLevel::CUDA.

    One renderer per stream; not thread-safe (as the reference's &mut self).
    """

    level = RendererLevel.CUDA

    def __init__(self, device: int = 0, options: RendererOptions | None = None):
        self._lib = _abi.lib()
        self._h = C.c_void_p()
        self.options = options or RendererOptions()
        o = self.options.to_c()
        _abi.check(self._lib.PFCUDARendererCreate(device, C.byref(o), C.byref(self._h)), "PFCUDARendererCreate")
        self._uploaded = None  # (scene id, epoch)

    def close(self) -> None:
        if self._h:
            self._lib.PFCUDARendererDestroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def set_stream(self, stream) -> None:
        """Run on a cudaStream_t (int handle or torch.cuda.Stream)."""
        h = getattr(stream, "cuda_stream", stream)
        _abi.check(self._lib.PFCUDARendererSetStream(self._h, C.c_void_p(h)), "PFCUDARendererSetStream")

    def set_options(self, options: RendererOptions) -> None:
        self.options = options
        o = options.to_c()
        _abi.check(self._lib.PFCUDARendererSetOptions(self._h, C.byref(o)), "PFCUDARendererSetOptions")

    def upload_scene(self, scene: Scene, force: bool = False) -> None:
        """UploadSceneD3D11: only when the scene id or epoch changed."""
        key = (scene.id, scene.epoch)
        if not force and self._uploaded == key:
            return
        d = scene.desc()
        _abi.check(self._lib.PFCUDASceneUpload(self._h, C.byref(d)), "PFCUDASceneUpload")
        self._uploaded = key

    def render(self, scene: Scene, options: BuildOptions | None = None, out=None,
               width: int | None = None, height: int | None = None, copy_image: bool = False):
        """Scene::build_and_render for the CUDA level: premultiplied RGBA8,
        row 0 at the top.  ``out`` may be a host numpy array or a CUDA tensor.
        ``copy_image``: a host ``out`` is written by one device-to-host copy
        after the composite (PF_MEMORY_HOST_COPY) instead of by the composite
        itself, which leaves the SMs to frames on other renderers."""
        self.upload_scene(scene)
        w, h = width or scene.width, height or scene.height
        if out is None:
            out = np.zeros((h, w, 4), np.uint8)
        p, mem = _ptr(out)
        if copy_image and mem == _abi.PF_MEMORY_HOST:
            mem = _abi.PF_MEMORY_HOST_COPY
        bo = (options or BuildOptions()).to_c()
        _abi.check(self._lib.PFCUDARenderScene(self._h, C.byref(bo), w, h, C.c_void_p(p), mem), "PFCUDARenderScene")
        return out

    def render_coverage(self, scene: Scene, options: BuildOptions | None = None, out=None,
                        width: int | None = None, height: int | None = None):
        """Single-channel FP32 render (SrcOver of paint alpha x coverage)."""
        self.upload_scene(scene)
        w, h = width or scene.width, height or scene.height
        if out is None:
            out = np.zeros((h, w), np.float32)
        p, mem = _ptr(out)
        bo = (options or BuildOptions()).to_c()
        _abi.check(self._lib.PFCUDARenderCoverage(self._h, C.byref(bo), w, h, C.c_void_p(p), mem),
                   "PFCUDARenderCoverage")
        return out

    def render_async(self, scene: Scene, out, options: BuildOptions | None = None,
                     width: int | None = None, height: int | None = None):
        """Enqueue a frame into a CUDA uint8 tensor without synchronising
        (capacity overflows surface in render_status())."""
        self.upload_scene(scene)
        w, h = width or scene.width, height or scene.height
        p, mem = _ptr(out)
        if mem != _abi.PF_MEMORY_DEVICE:
            raise ValueError("render_async needs a device output buffer")
        bo = (options or BuildOptions()).to_c()
        _abi.check(self._lib.PFCUDARenderSceneAsync(self._h, C.byref(bo), w, h, C.c_void_p(p)),
                   "PFCUDARenderSceneAsync")
        return out

    def render_status(self) -> tuple[int, int]:
        """(status code, needed capacity) of the frames enqueued since the last call."""
        n = C.c_uint64()
        code = self._lib.PFCUDARenderStatus(self._h, C.byref(n))
        return code, n.value

    def set_profiling(self, enable: bool) -> None:
        _abi.check(self._lib.PFCUDASetProfiling(self._h, 1 if enable else 0), "PFCUDASetProfiling")

    def stage_times(self) -> dict:
        """Per-stage milliseconds of the last profiled frame (synchronises)."""
        a = (C.c_float * _abi.PF_CUDA_STAGE_COUNT)()
        _abi.check(self._lib.PFCUDAGetStageTimes(self._h, a, _abi.PF_CUDA_STAGE_COUNT), "PFCUDAGetStageTimes")
        return {n: float(a[i]) for i, n in enumerate(_abi.STAGE_NAMES)}

    # --- batches -------------------------------------------------------------
    def upload_batch(self, batch, force: bool = False) -> None:
        """PFCUDASceneUploadBatch: many independent scenes at once."""
        key = ("batch", batch.key)
        if not force and self._uploaded == key:
            return
        _abi.check(self._lib.PFCUDASceneUploadBatch(self._h, *batch.upload_args()), "PFCUDASceneUploadBatch")
        self._uploaded = key

    def render_batch(self, batch, out, fmt: int = _abi.PF_CUDA_FORMAT_RGBA8, first: int = 0,
                     count: int | None = None, options: BuildOptions | None = None, sync: bool = True):
        """Render scenes [first, first+count) of `batch` into device tensor `out`."""
        self.upload_batch(batch)
        count = len(batch) - first if count is None else count
        p, mem = _ptr(out)
        if mem != _abi.PF_MEMORY_DEVICE:
            raise ValueError("batched frames render into device memory")
        bo = (options or BuildOptions()).to_c()
        fn = self._lib.PFCUDARenderBatch if sync else self._lib.PFCUDARenderBatchAsync
        _abi.check(fn(self._h, C.byref(bo), first, count, fmt, C.c_void_p(p)), "PFCUDARenderBatch")
        return out

    def graph_capture(self, batch, out, fmt: int = _abi.PF_CUDA_FORMAT_RGBA8, first: int = 0,
                      count: int | None = None, options: BuildOptions | None = None) -> None:
        """Capture one frame of the batch range into a CUDA graph (batch=None:
        the scene(s) already uploaded, with the targets of their last frame)."""
        if batch is not None:
            self.upload_batch(batch)
            count = len(batch) - first if count is None else count
        elif count is None:
            count = 1
        p, _ = _ptr(out)
        bo = (options or BuildOptions()).to_c()
        _abi.check(self._lib.PFCUDAGraphCapture(self._h, C.byref(bo), first, count, fmt, C.c_void_p(p)),
                   "PFCUDAGraphCapture")

    def graph_launch(self) -> None:
        _abi.check(self._lib.PFCUDAGraphLaunch(self._h), "PFCUDAGraphLaunch")

    def graph_release(self) -> None:
        _abi.check(self._lib.PFCUDAGraphRelease(self._h), "PFCUDAGraphRelease")

    def get_tuning(self) -> dict:
        t = _abi.PFCUDATuning()
        _abi.check(self._lib.PFCUDAGetTuning(self._h, C.byref(t)), "PFCUDAGetTuning")
        return {k: getattr(t, k) for k, _ in t._fields_}

    def set_tuning(self, **kw) -> None:
        cur = self.get_tuning()
        cur.update(kw)
        t = _abi.PFCUDATuning(**cur)
        _abi.check(self._lib.PFCUDASetTuning(self._h, C.byref(t)), "PFCUDASetTuning")

    def autotune(self, batch, out, fmt: int = _abi.PF_CUDA_FORMAT_RGBA8, first: int = 0,
                 count: int | None = None, repeats: int = 3, options: BuildOptions | None = None) -> dict:
        """Time candidate launch shapes on this batch range; keep the fastest."""
        self.upload_batch(batch)
        count = len(batch) - first if count is None else count
        p, _ = _ptr(out)
        bo = (options or BuildOptions()).to_c()
        t = _abi.PFCUDATuning()
        _abi.check(self._lib.PFCUDAAutotune(self._h, C.byref(bo), first, count, fmt, C.c_void_p(p), repeats,
                                            C.byref(t)), "PFCUDAAutotune")
        return {k: getattr(t, k) for k, _ in t._fields_}

    # --- differentiable frames ----------------------------------------------
    def set_points(self, points) -> None:
        """PFCUDASetPoints: replace every uploaded point ([N, 2] float32, host
        array or CUDA tensor, batch order) without re-uploading the scene."""
        p, mem = _ptr(points)
        n = int(points.shape[0])
        _abi.check(self._lib.PFCUDASetPoints(self._h, C.c_void_p(p), n, mem), "PFCUDASetPoints")

    def render_diff(self, out, first: int = 0, count: int = 1, width: int = 0, height: int = 0, alpha=None,
                    options: BuildOptions | None = None, sync: bool = True):
        """PFCUDARenderDiff (sync) or PFCUDARenderDiffAsync into the float32
        CUDA tensor `out`.  `alpha`: CUDA float32 tensor, one value per draw
        path of the uploaded batch (None: paint alpha).  width/height > 0 place
        scenes without a target into a width x height image."""
        p, mem = _ptr(out)
        if mem != _abi.PF_MEMORY_DEVICE:
            raise ValueError("differentiable frames render into device memory")
        ap = 0
        if alpha is not None:
            ap, amem = _ptr(alpha)
            if amem != _abi.PF_MEMORY_DEVICE:
                raise ValueError("alpha must be a CUDA tensor")
        bo = (options or BuildOptions()).to_c()
        fn = self._lib.PFCUDARenderDiff if sync else self._lib.PFCUDARenderDiffAsync
        _abi.check(fn(self._h, C.byref(bo), first, count, width, height, C.c_void_p(ap) if ap else None,
                      C.c_void_p(p)), "PFCUDARenderDiff")
        return out

    def backward(self, d_image, d_points, d_alpha=None) -> None:
        """PFCUDABackward of the last render_diff: writes dL/dpoints ([N, 2]
        CUDA float32) and dL/dalpha (per draw path, optional)."""
        gi, m0 = _ptr(d_image)
        gp, m1 = _ptr(d_points)
        ga = 0
        if d_alpha is not None:
            ga, m2 = _ptr(d_alpha)
            if m2 != _abi.PF_MEMORY_DEVICE:
                raise ValueError("d_alpha must be a CUDA tensor")
        if m0 != _abi.PF_MEMORY_DEVICE or m1 != _abi.PF_MEMORY_DEVICE:
            raise ValueError("the adjoint works on CUDA tensors")
        _abi.check(self._lib.PFCUDABackward(self._h, C.c_void_p(gi), C.c_void_p(gp), C.c_void_p(ga) if ga else None),
                   "PFCUDABackward")

    def stroke_to_fill_buffers(self, items):
        """PFCUDAStrokeToFill over [(Outline, StrokeStyle)] (PFCUDAStrokeToFillDashed
        when an item is (Outline, StrokeStyle, dashes, dash_offset) with a
        non-empty pattern): the stroked outlines as (points (N, 2) float32,
        flags (N,) uint8, contour_starts, outline_starts)."""
        from .stroke import StrokeBatch
        b = StrokeBatch(items)
        d = b.desc()
        dd = b.dash_desc() if b.dashed else None
        cap_p = max(64, 8 * len(b.points) + 64 * b.contour_count)
        cap_c = 2 * b.contour_count
        for _ in range(2):
            pts = np.zeros((cap_p, 2), np.float32)
            flags = np.zeros((cap_p,), np.uint8)
            cs = np.zeros((cap_c + 1,), np.uint32)
            os_ = np.zeros((b.outline_count + 1,), np.uint32)
            o = _abi.PFCUDAStrokeOutput()
            o.points, o.point_flags = pts.ctypes.data, flags.ctypes.data
            o.contour_starts, o.outline_starts = cs.ctypes.data, os_.ctypes.data
            o.point_capacity, o.contour_capacity = cap_p, cap_c
            o.memory = _abi.PF_MEMORY_HOST
            if dd is None:
                rc = self._lib.PFCUDAStrokeToFill(self._h, C.byref(d), C.byref(o))
            else:
                rc = self._lib.PFCUDAStrokeToFillDashed(self._h, C.byref(d), C.byref(dd), C.byref(o))
            if rc == _abi.PF_CUDA_ERR_CAPACITY and (o.point_count > cap_p or o.contour_count > cap_c):
                cap_p, cap_c = int(o.point_count), int(o.contour_count)
                continue
            _abi.check(rc, "PFCUDAStrokeToFill")
            n, nc = int(o.point_count), int(o.contour_count)
            return pts[:n], flags[:n], cs[:nc + 1], os_
        raise RuntimeError("PFCUDAStrokeToFill: capacity did not converge")

    def dash_buffers(self, items):
        """PFCUDADashOutlines over [(Outline, dashes, dash_offset)]: the dashed
        outlines as (points (N, 2) float32, flags (N,) uint8, contour_starts,
        contour_closed, outline_starts)."""
        from .stroke import StrokeBatch
        b = StrokeBatch([(ol, None, dashes, offset) for ol, dashes, offset in items])
        d, dd = b.desc(), b.dash_desc()
        cap_p = max(64, 4 * len(b.points))
        cap_c = max(16, 4 * b.contour_count)
        for _ in range(2):
            pts = np.zeros((cap_p, 2), np.float32)
            flags = np.zeros((cap_p,), np.uint8)
            cs = np.zeros((cap_c + 1,), np.uint32)
            closed = np.zeros((max(1, cap_c),), np.uint8)
            os_ = np.zeros((b.outline_count + 1,), np.uint32)
            o = _abi.PFCUDAOutlineOutput()
            o.points, o.point_flags = pts.ctypes.data, flags.ctypes.data
            o.contour_starts, o.contour_closed, o.outline_starts = cs.ctypes.data, closed.ctypes.data, os_.ctypes.data
            o.point_capacity, o.contour_capacity = cap_p, cap_c
            o.memory = _abi.PF_MEMORY_HOST
            rc = self._lib.PFCUDADashOutlines(self._h, C.byref(d), C.byref(dd), C.byref(o))
            if rc == _abi.PF_CUDA_ERR_CAPACITY and (o.point_count > cap_p or o.contour_count > cap_c):
                cap_p, cap_c = int(o.point_count), int(o.contour_count)
                continue
            _abi.check(rc, "PFCUDADashOutlines")
            n, nc = int(o.point_count), int(o.contour_count)
            return pts[:n], flags[:n], cs[:nc + 1], closed[:nc], os_
        raise RuntimeError("PFCUDADashOutlines: capacity did not converge")

    def dash_outlines(self, items):
        """OutlineDash (content/src/dash.rs:18-152) for many outlines at once on
        the GPU: [(Outline, dashes, dash_offset)] -> [Outline] (dashed contours
        open; an outline with an empty pattern unchanged)."""
        from .stroke import outlines_from_buffers
        pts, flags, cs, closed, os_ = self.dash_buffers(items)
        return outlines_from_buffers(pts, flags, cs, os_, closed)

    def stroke_to_fill(self, items):
        """OutlineStrokeToFill (content/src/stroke.rs:24-190) for many outlines at
        once on the GPU: [(Outline, StrokeStyle)] -> [Outline] of closed contours."""
        from .stroke import outlines_from_buffers
        return outlines_from_buffers(*self.stroke_to_fill_buffers(items))

    def stats(self) -> RenderStats:
        s = _abi.PFCUDARenderStats()
        _abi.check(self._lib.PFCUDAGetStats(self._h, C.byref(s)), "PFCUDAGetStats")
        return RenderStats(**{k: getattr(s, k) for k, _ in s._fields_})

    def read_records(self, scene: Scene) -> dict:
        """Fill / tile / clip records and the z-buffer of the last frame."""
        st = self.stats()
        F, T = st.fill_count, st.tile_count
        P = len(scene.clip_paths) + len(scene.draw_paths)
        fills = np.zeros((F,), _FILL)
        fill_tile = np.zeros((F,), np.uint32)
        tiles = np.zeros((T,), _TILE)
        clips = np.zeros((T,), _CLIP)
        offs = np.zeros((P + 1,), np.uint32)
        rects = np.zeros((P + 1,), _RECT)
        z = np.zeros((max(st.screen_tile_count, 1),), np.int32)
        _abi.check(self._lib.PFCUDAReadRecords(self._h, fills.ctypes.data, fill_tile.ctypes.data, F,
                                               tiles.ctypes.data, T, offs.ctypes.data, rects.ctypes.data, P + 1,
                                               clips.ctypes.data, z.ctypes.data, len(z)), "PFCUDAReadRecords")
        return dict(fills=fills, fill_tile=fill_tile, tiles=tiles, clips=clips, path_tile_offsets=offs,
                    path_tile_rects=rects[:P], z_buffer=z[:st.screen_tile_count])

    def read_masks(self):
        """(raw alpha masks [A,16,16], resolved coverage per path tile [T,16,16]) of the last frame."""
        st = self.stats()
        a = np.zeros((max(st.alpha_tile_count, 1), 16, 16), np.float32)
        t = np.zeros((max(st.tile_count, 1), 16, 16), np.float32)
        _abi.check(self._lib.PFCUDAReadMasks(self._h, a.ctypes.data, st.alpha_tile_count, t.ctypes.data,
                                             st.tile_count), "PFCUDAReadMasks")
        return a[:st.alpha_tile_count], t[:st.tile_count]
