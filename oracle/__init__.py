"""The parity oracle — TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.

A CPU restatement (pf_oracle.cpp) of the reference's CPU tiler plus an FP64
evaluation of its coverage formula, mask resolve and composite.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, and only as
the checker or the timed CPU baseline.

Parity status: the tiler is pinned by hand-derived known-answer cases only
(the reference has no tiler tests and its Rust cannot be built here); the
coverage formula is pinned by the reference's own area LUT
(tests/golden/area_lut.*).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "pf_oracle.cpp")
# The seeded scene generators (pathfinder_gb300/csrc/pf_scenes.cpp, host code)
# are compiled in too, so that the CPU baseline can build its input scenes
# without loading the CUDA library.
SCENES_SRC = os.path.join(ROOT, "pathfinder_gb300", "csrc", "pf_scenes.cpp")
SRCS = [SRC, os.path.join(HERE, "pf_oracle_stroke.cpp"), SCENES_SRC]
LIB_PATH = os.path.join(HERE, "libpforacle.so")

CXXFLAGS = ["-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-Wall"]


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no FMA contraction: SSE op order)."""
    if not force and os.path.exists(LIB_PATH) and all(os.path.getmtime(LIB_PATH) >= os.path.getmtime(s)
                                                       for s in SRCS):
        return LIB_PATH
    cmd = ["g++"] + CXXFLAGS + ["-I", os.path.join(ROOT, "include"), "-o", LIB_PATH] + SRCS + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB_PATH


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(LIB_PATH)
        l.pfo_build.restype = C.c_void_p
        l.pfo_build.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_uint64, C.c_int32]
        l.pfo_free.argtypes = [C.c_void_p]
        l.pfo_counts.argtypes = [C.c_void_p, C.c_void_p]
        l.pfo_fills.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        l.pfo_tiles.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        l.pfo_zbuffer.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        l.pfo_masks.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        l.pfo_mask_error.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        l.pfo_render.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                 C.c_int]
        l.pfo_render_glyphs.restype = C.c_int32
        l.pfo_render_glyphs.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_int, C.c_void_p, C.c_int]
        l.pfo_cpu_frame.restype = C.c_double
        l.pfo_cpu_frame.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        l.pfo_area.restype = C.c_double
        l.pfo_area.argtypes = [C.c_double, C.c_double]
        l.pfo_fill_coverage.argtypes = [C.c_void_p, C.c_void_p]
        l.pfo_area_lut_value.restype = C.c_uint8
        l.pfo_area_lut_value.argtypes = [C.c_int, C.c_int, C.c_int]
        l.pfo_gradient_sample.restype = C.c_int32
        l.pfo_gradient_sample.argtypes = [C.c_void_p, C.c_float, C.c_void_p]
        l.pfo_round_f16.restype = C.c_float
        l.pfo_round_f16.argtypes = [C.c_float]
        l.pfo_sse_cvt.restype = C.c_int32
        l.pfo_sse_cvt.argtypes = [C.c_float]
        l.pfo_diff_build.restype = C.c_void_p
        l.pfo_diff_build.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        l.pfo_diff_free.argtypes = [C.c_void_p]
        l.pfo_diff_info.argtypes = [C.c_void_p, C.c_void_p]
        l.pfo_diff_render.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]
        l.pfo_diff_grad.restype = C.c_int32
        l.pfo_diff_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        _lib = l
    return _lib


def generate_scene(workload: int, seed: int = 1, scale: float = 1.0, **kw):
    """The seeded scene generator compiled into this library (the same source
    as the package's libpfscenes.so), for CPU-only runs that must not load the
    CUDA library."""
    from pathfinder_gb300 import _abi
    from pathfinder_gb300.scene import generate_scene as gen
    return gen(workload, seed=seed, scale=scale, lib=_abi.bind_scene_generator(lib()), **kw)


def _dtypes():
    from pathfinder_gb300 import _abi
    return _abi.record_dtypes()


def _opts(build_options):
    if build_options is None:
        return None
    o = build_options.to_c()
    return o


class OracleFrame:
    """One build of a scene by the CPU tiler restatement."""

    def __init__(self, scene, build_options=None, threads: int = 0, dda_limit: int = 0, d3d11: bool = False):
        """d3d11: the D3D11 level's tiling (uniform dicing, unclipped
        truncating bins) in place of the CPU tiler's."""
        L = lib()
        self._scene = scene
        self._desc = scene.desc()
        self._bo = _opts(build_options)
        threads = threads or (os.cpu_count() or 1)
        self.threads = threads
        h = L.pfo_build(C.byref(self._desc), C.byref(self._bo) if self._bo is not None else None, threads,
                        dda_limit, 1 if d3d11 else 0)
        if not h:
            raise ValueError("oracle rejected the scene")
        self._h = h
        c = np.zeros((8,), np.uint64)
        L.pfo_counts(h, c.ctypes.data)
        (self.path_count, self.tile_count, self.fill_count, self.alpha_tile_count, self.line_count,
         self.screen_tile_count, limit, self.clip_path_count) = [int(v) for v in c]
        self.limit_hit = bool(limit)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().pfo_free(self._h)
            self._h = None

    def fills(self):
        fill, *_ = _dtypes()
        f = np.zeros((self.fill_count,), fill)
        t = np.zeros((self.fill_count,), np.uint32)
        lib().pfo_fills(self._h, f.ctypes.data, t.ctypes.data)
        return f, t

    def tiles(self):
        _, tile, clip, _, rect = _dtypes()
        tiles = np.zeros((self.tile_count,), tile)
        clips = np.zeros((self.tile_count,), clip)
        offs = np.zeros((self.path_count + 1,), np.uint32)
        rects = np.zeros((self.path_count,), rect)
        lib().pfo_tiles(self._h, tiles.ctypes.data, clips.ctypes.data, offs.ctypes.data, rects.ctypes.data, None)
        return tiles, clips, offs, rects

    def zbuffer(self):
        z = np.zeros((self.screen_tile_count,), np.int32)
        lib().pfo_zbuffer(self._h, z.ctypes.data, None)
        return z

    def masks(self):
        """(raw alpha masks [A,16,16] FP64, resolved coverage per path tile [T,16,16] FP64)."""
        a = np.zeros((self.alpha_tile_count, 16, 16), np.float64)
        t = np.zeros((self.tile_count, 16, 16), np.float64)
        lib().pfo_masks(self._h, a.ctypes.data, t.ctypes.data, self.threads)
        return a, t

    def mask_error(self, gpu_alpha=None, gpu_tile=None):
        """Largest |gpu - oracle| of float32 raw alpha masks [A,16,16] and of
        resolved tile coverage [T,16,16], computed tile by tile against the
        FP64 values (no FP64 copy of the arrays).  Returns ((raw, tile),
        (alpha tile, path tile) of the largest errors)."""
        ga = None if gpu_alpha is None else np.ascontiguousarray(gpu_alpha, np.float32)
        gt = None if gpu_tile is None else np.ascontiguousarray(gpu_tile, np.float32)
        if ga is not None and ga.size != self.alpha_tile_count * 256:
            raise ValueError("alpha mask count differs from the oracle's")
        if gt is not None and gt.size != self.tile_count * 256:
            raise ValueError("tile count differs from the oracle's")
        err = np.zeros((2,), np.float64)
        where = np.zeros((2,), np.uint64)
        lib().pfo_mask_error(self._h, ga.ctypes.data if ga is not None else None,
                             gt.ctypes.data if gt is not None else None, err.ctypes.data, where.ctypes.data,
                             self.threads)
        return (float(err[0]), float(err[1])), (int(where[0]), int(where[1]))

    def render(self, width: int, height: int, background=None, channels: int = 4):
        from pathfinder_gb300 import _abi
        bg = None
        if background is not None:
            bg = _abi.PFColorF(*background)
        if channels == 4:
            out = np.zeros((height, width, 4), np.uint8)
            f64 = np.zeros((height, width, 4), np.float64)
        else:
            out = np.zeros((height, width), np.uint8)
            f64 = np.zeros((height, width), np.float64)
        lib().pfo_render(self._h, width, height, C.byref(bg) if bg is not None else None, channels,
                         out.ctypes.data, f64.ctypes.data, self.threads)
        return out, f64


class DiffOracle:
    """FP64 differentiable frame of a scene and its adjoint, with each curve's
    subdivision fixed by the FP32 flattening of the scene's own points (the
    checker of the CUDA level's PFCUDARenderDiff / PFCUDABackward)."""

    def __init__(self, scene, width: int, height: int, build_options=None):
        L = lib()
        self._scene = scene
        self._desc = scene.desc()
        self._bo = _opts(build_options)
        h = L.pfo_diff_build(C.byref(self._desc), C.byref(self._bo) if self._bo is not None else None, width,
                             height)
        if not h:
            raise ValueError("oracle rejected the scene")
        self._h = h
        self.width, self.height = width, height
        info = np.zeros((5,), np.uint64)
        L.pfo_diff_info(h, info.ctypes.data)
        self.point_count, self.clip_path_count, self.draw_path_count, self.line_count, limit = [int(v) for v in info]
        self.limit_hit = bool(limit)
        self.points = np.asarray(scene.points, np.float64).reshape(-1, 2).copy()
        self.alpha = scene.draw_paths["paint"][:, 3].astype(np.float64) / 255.0

    def __del__(self):
        if getattr(self, "_h", None):
            lib().pfo_diff_free(self._h)
            self._h = None

    def render(self, points=None, alpha=None, background: float = 0.0) -> np.ndarray:
        p = np.ascontiguousarray(self.points if points is None else points, np.float64).reshape(-1, 2)
        a = np.ascontiguousarray(self.alpha if alpha is None else alpha, np.float64)
        if p.shape[0] != self.point_count or a.shape[0] != self.draw_path_count:
            raise ValueError("points / alpha do not match the scene")
        img = np.zeros((self.height, self.width), np.float64)
        lib().pfo_diff_render(self._h, p.ctypes.data, a.ctypes.data, float(background), img.ctypes.data)
        return img

    def grad(self, d_image) -> tuple[np.ndarray, np.ndarray]:
        """(dL/dpoints [N,2], dL/dalpha [draw paths]) of the last render."""
        g = np.ascontiguousarray(d_image, np.float64)
        if g.shape != (self.height, self.width):
            raise ValueError("d_image has the wrong shape")
        dp = np.zeros((self.point_count, 2), np.float64)
        da = np.zeros((self.draw_path_count,), np.float64)
        if lib().pfo_diff_grad(self._h, g.ctypes.data, dp.ctypes.data, da.ctypes.data) != 0:
            raise RuntimeError("render before grad")
        return dp, da


def render_glyphs(atlas, threads: int = 0) -> np.ndarray:
    """Every glyph of an atlas scene rendered as its own scene (its path alone,
    view box = its cell) into its cell of one R8 image, FP64 coverage rounded
    to u8: what a batch of glyph scenes writes."""
    if atlas.cells is None:
        raise ValueError("the scene has no glyph cells")
    d = atlas.desc()
    cells = np.ascontiguousarray(atlas.cells)
    out = np.zeros((atlas.height, atlas.width), np.uint8)
    rc = lib().pfo_render_glyphs(C.byref(d), cells.ctypes.data, len(cells), atlas.width, atlas.height,
                                 out.ctypes.data, threads or (os.cpu_count() or 1))
    if rc != 0:
        raise ValueError("oracle rejected the atlas scene")
    return out


def cpu_frame(scene, width: int, height: int, threads: int = 0, build_options=None, want_image: bool = False):
    """Time one CPU-baseline frame (tiling + FP32 coverage + composite).
    Returns (seconds, image or None, counts)."""
    L = lib()
    d = scene.desc()
    bo = _opts(build_options)
    out = np.zeros((height, width, 4), np.uint8) if want_image else None
    counts = np.zeros((8,), np.uint64)
    secs = L.pfo_cpu_frame(C.byref(d), C.byref(bo) if bo is not None else None, width, height,
                           threads or (os.cpu_count() or 1), out.ctypes.data if out is not None else None,
                           counts.ctypes.data)
    return secs, out, counts


def area(y: float, dydx: float) -> float:
    return lib().pfo_area(y, dydx)


def fill_coverage(seg) -> np.ndarray:
    m = np.zeros((16, 16), np.float64)
    s = (C.c_uint16 * 4)(*[int(v) for v in seg])
    lib().pfo_fill_coverage(s, m.ctypes.data)
    return m


def dash(stroke_input, dash_input):
    """The oracle's OutlineDash of a host-memory PFCUDAStrokeInput with a
    host-memory PFCUDADashInput: (points (N, 2) float32, flags (N,) uint8,
    contour_starts, contour_closed, outline_starts, step_limit_hit)."""
    L = lib()
    L.pfo_dash.restype = C.c_void_p
    L.pfo_dash.argtypes = [C.c_void_p, C.c_void_p]
    L.pfo_dash_counts.argtypes = [C.c_void_p, C.c_void_p]
    L.pfo_dash_read.argtypes = [C.c_void_p] * 6
    L.pfo_dash_free.argtypes = [C.c_void_p]
    h = L.pfo_dash(C.byref(stroke_input), C.byref(dash_input))
    if not h:
        raise ValueError("oracle rejected the dash input")
    try:
        n = np.zeros((3,), np.uint64)
        L.pfo_dash_counts(h, n.ctypes.data)
        npts, nc = int(n[0]), int(n[1])
        pts = np.zeros((npts, 2), np.float32)
        flags = np.zeros((npts,), np.uint8)
        cs = np.zeros((nc + 1,), np.uint32)
        closed = np.zeros((nc,), np.uint8)
        os_ = np.zeros((stroke_input.outline_count + 1,), np.uint32)
        L.pfo_dash_read(h, pts.ctypes.data, flags.ctypes.data, cs.ctypes.data, closed.ctypes.data, os_.ctypes.data)
        return pts, flags, cs, closed, os_, bool(n[2])
    finally:
        L.pfo_dash_free(h)


def area_lut_value(u: int, v: int, k: int) -> int:
    """The reference LUT texel (u, v) channel k, computed in f32 by the oracle."""
    return int(lib().pfo_area_lut_value(u, v, k))


def sse_cvt(x: float) -> int:
    return int(lib().pfo_sse_cvt(x))


def stroke(stroke_input):
    """The oracle's stroke-to-fill of a host-memory PFCUDAStrokeInput:
    (points (N, 2) float32, flags (N,) uint8, contour_starts, outline_starts,
    depth_limit_hit)."""
    L = lib()
    L.pfo_stroke.restype = C.c_void_p
    L.pfo_stroke.argtypes = [C.c_void_p]
    L.pfo_stroke_counts.argtypes = [C.c_void_p, C.c_void_p]
    L.pfo_stroke_read.argtypes = [C.c_void_p] * 5
    L.pfo_stroke_free.argtypes = [C.c_void_p]
    h = L.pfo_stroke(C.byref(stroke_input))
    if not h:
        raise ValueError("oracle rejected the stroke input")
    try:
        n = np.zeros((3,), np.uint64)
        L.pfo_stroke_counts(h, n.ctypes.data)
        npts, nc = int(n[0]), int(n[1])
        pts = np.zeros((npts, 2), np.float32)
        flags = np.zeros((npts,), np.uint8)
        cs = np.zeros((nc + 1,), np.uint32)
        os_ = np.zeros((stroke_input.outline_count + 1,), np.uint32)
        L.pfo_stroke_read(h, pts.ctypes.data, flags.ctypes.data, cs.ctypes.data, os_.ctypes.data)
        return pts, flags, cs, os_, bool(n[2])
    finally:
        L.pfo_stroke_free(h)
