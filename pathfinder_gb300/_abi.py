"""ctypes declarations of the C ABI in include/pathfinder_cuda.h and
include/pathfinder_cuda_scenes.h.

The library is loaded from the package directory; there is no fallback: if
``libpathfinder_cuda.so`` is missing or cannot be loaded, importing the
renderer raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpathfinder_cuda.so")

PF_CUDA_OK = 0
PF_CUDA_ERR_INVALID = 1
PF_CUDA_ERR_CAPACITY = 2
PF_CUDA_ERR_LAUNCH = 3
PF_CUDA_ERR_NO_DEVICE = 4
PF_CUDA_ERR_LIMIT = 5
PF_CUDA_ERR_NO_SCENE = 6

PF_MEMORY_HOST = 0
PF_MEMORY_DEVICE = 1
PF_MEMORY_HOST_COPY = 2  # frame outputs: host memory written by one device-to-host copy

PF_CUDA_RENDERER_D3D11_SEMANTICS = 0x1

# BlendMode (content/src/effects.rs:99-160), SrcOver first
BLEND_MODES = ["src_over", "clear", "copy", "src_in", "src_out", "src_atop", "dest_in", "dest_out",
               "dest_over", "dest_atop", "xor", "lighter", "darken", "lighten", "multiply", "screen",
               "hard_light", "overlay", "color_dodge", "color_burn", "soft_light", "difference",
               "exclusion", "hue", "saturation", "color", "luminosity"]
PF_BLEND_MODE_COUNT = len(BLEND_MODES)

PF_GRADIENT_LINEAR = 0
PF_GRADIENT_RADIAL = 1
PF_GRADIENT_WRAP_CLAMP = 0
PF_GRADIENT_WRAP_REPEAT = 1

PF_PATTERN_REPEAT_X = 0x1
PF_PATTERN_REPEAT_Y = 0x2
PF_PATTERN_NO_SMOOTHING = 0x4
PF_PATTERN_FILTER_NONE = 0
PF_PATTERN_FILTER_BLUR_X = 1
PF_PATTERN_FILTER_BLUR_Y = 2
PF_PATTERN_FILTER_COLOR_MATRIX = 3

PF_LINE_CAP_BUTT = 0
PF_LINE_CAP_SQUARE = 1
PF_LINE_CAP_ROUND = 2
PF_LINE_JOIN_MITER = 0
PF_LINE_JOIN_BEVEL = 1
PF_LINE_JOIN_ROUND = 2

PF_SCENE_STARS_512 = 1
PF_SCENE_SVG_4K = 2
PF_SCENE_GLYPH_ATLAS = 3
PF_SCENE_CUBIC_1K = 4
PF_SCENE_EDGE_CASES = 5

PF_CUDA_STAGE_COUNT = 9
STAGE_NAMES = ["bound", "flatten", "bin_count", "scans", "bin_emit", "propagate", "visibility", "fill", "composite"]


class PFVector2F(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class PFVector2I(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32)]


class PFRectF(C.Structure):
    _fields_ = [("origin", PFVector2F), ("lower_right", PFVector2F)]


class PFRectI(C.Structure):
    _fields_ = [("origin", PFVector2I), ("lower_right", PFVector2I)]


class PFColorU(C.Structure):
    _fields_ = [("r", C.c_uint8), ("g", C.c_uint8), ("b", C.c_uint8), ("a", C.c_uint8)]


class PFColorF(C.Structure):
    _fields_ = [("r", C.c_float), ("g", C.c_float), ("b", C.c_float), ("a", C.c_float)]


class PFTransform2F(C.Structure):
    _fields_ = [("m00", C.c_float), ("m01", C.c_float), ("m10", C.c_float), ("m11", C.c_float),
                ("vector", PFVector2F)]


class PFCUDAPath(C.Structure):
    _fields_ = [("first_contour", C.c_uint32), ("contour_count", C.c_uint32), ("paint", PFColorU),
                ("clip_path", C.c_int32), ("fill_rule", C.c_uint8), ("blend_mode", C.c_uint8),
                ("overlay", C.c_uint16)]


class PFCUDAColorStop(C.Structure):
    _fields_ = [("offset", C.c_float), ("color", PFColorU)]


class PFCUDAGradient(C.Structure):
    _fields_ = [("kind", C.c_int32), ("wrap", C.c_int32), ("from_", PFVector2F), ("to", PFVector2F),
                ("radius0", C.c_float), ("radius1", C.c_float), ("transform", PFTransform2F),
                ("stops", C.c_void_p), ("stop_count", C.c_uint32), ("reserved", C.c_uint32)]


class PFCUDAPattern(C.Structure):
    _fields_ = [("pixels", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("transform", PFTransform2F), ("flags", C.c_uint32), ("filter", C.c_int32),
                ("blur_sigma", C.c_float), ("color_matrix", C.c_float * 20)]


class PFCUDASceneDesc(C.Structure):
    _fields_ = [("points", C.c_void_p), ("point_flags", C.c_void_p), ("contour_starts", C.c_void_p),
                ("clip_paths", C.c_void_p), ("draw_paths", C.c_void_p),
                ("point_count", C.c_uint32), ("contour_count", C.c_uint32),
                ("clip_path_count", C.c_uint32), ("draw_path_count", C.c_uint32),
                ("view_box", PFRectF), ("memory", C.c_int32),
                ("gradients", C.c_void_p), ("gradient_count", C.c_uint32),
                ("patterns", C.c_void_p), ("pattern_count", C.c_uint32)]


class PFCUDAStrokeStyle(C.Structure):
    _fields_ = [("line_width", C.c_float), ("line_cap", C.c_int32), ("line_join", C.c_int32),
                ("miter_limit", C.c_float)]


class PFCUDAStrokeInput(C.Structure):
    _fields_ = [("points", C.c_void_p), ("point_flags", C.c_void_p), ("contour_starts", C.c_void_p),
                ("contour_closed", C.c_void_p), ("outline_starts", C.c_void_p), ("styles", C.c_void_p),
                ("point_count", C.c_uint32), ("contour_count", C.c_uint32), ("outline_count", C.c_uint32),
                ("memory", C.c_int32)]


class PFCUDAStrokeOutput(C.Structure):
    _fields_ = [("points", C.c_void_p), ("point_flags", C.c_void_p), ("contour_starts", C.c_void_p),
                ("outline_starts", C.c_void_p), ("point_capacity", C.c_uint64),
                ("contour_capacity", C.c_uint64), ("point_count", C.c_uint64), ("contour_count", C.c_uint64),
                ("memory", C.c_int32)]


class PFCUDADashInput(C.Structure):
    _fields_ = [("dashes", C.c_void_p), ("dash_starts", C.c_void_p), ("offsets", C.c_void_p)]


class PFCUDAOutlineOutput(C.Structure):
    _fields_ = [("points", C.c_void_p), ("point_flags", C.c_void_p), ("contour_starts", C.c_void_p),
                ("contour_closed", C.c_void_p), ("outline_starts", C.c_void_p), ("point_capacity", C.c_uint64),
                ("contour_capacity", C.c_uint64), ("point_count", C.c_uint64), ("contour_count", C.c_uint64),
                ("memory", C.c_int32)]


class PFCUDABuildOptions(C.Structure):
    _fields_ = [("transform", PFTransform2F), ("has_transform", C.c_int32)]


class PFCUDARendererOptions(C.Structure):
    _fields_ = [("background_color", PFColorF), ("has_background_color", C.c_int32), ("flags", C.c_int32)]


class PFCUDARenderStats(C.Structure):
    _fields_ = [("path_count", C.c_uint64), ("segment_count", C.c_uint64), ("line_count", C.c_uint64),
                ("fill_count", C.c_uint64), ("tile_count", C.c_uint64), ("alpha_tile_count", C.c_uint64),
                ("visible_tile_count", C.c_uint64), ("screen_tile_count", C.c_uint64),
                ("status", C.c_uint64), ("gpu_time_ms", C.c_double), ("kernel_launches", C.c_uint64),
                ("mask_tile_count", C.c_uint64), ("mask_fill_count", C.c_uint64)]


class PFCUDAFill(C.Structure):
    _fields_ = [("from_x", C.c_uint16), ("from_y", C.c_uint16), ("to_x", C.c_uint16), ("to_y", C.c_uint16),
                ("emission_index", C.c_uint32)]


class PFCUDATile(C.Structure):
    _fields_ = [("tile_x", C.c_int16), ("tile_y", C.c_int16), ("alpha_tile_id", C.c_uint32),
                ("path_id", C.c_uint32), ("color", C.c_uint16), ("ctrl", C.c_uint8), ("backdrop", C.c_int8)]


class PFCUDAClip(C.Structure):
    _fields_ = [("dest_tile_id", C.c_uint32), ("dest_backdrop", C.c_int32), ("src_tile_id", C.c_uint32),
                ("src_backdrop", C.c_int32)]


class PFCUDASceneTarget(C.Structure):
    _fields_ = [("out_offset", C.c_uint64), ("pitch", C.c_int32), ("origin_x", C.c_int32), ("origin_y", C.c_int32),
                ("clip", PFRectI)]


class PFCUDATuning(C.Structure):
    _fields_ = [("flatten_threads", C.c_int32), ("bin_threads", C.c_int32), ("bin_blocks_per_sm", C.c_int32),
                ("composite_warps", C.c_int32), ("composite_batch", C.c_int32), ("mask_stage_fills", C.c_int32)]


PF_CUDA_FORMAT_RGBA8 = 0
PF_CUDA_FORMAT_R8 = 1
PF_CUDA_FORMAT_F32 = 2


class PFCUDASceneParams(C.Structure):
    _fields_ = [("workload", C.c_int32), ("seed", C.c_uint64), ("scale", C.c_double),
                ("jitter_sigma", C.c_double), ("jitter_seed", C.c_uint64), ("width", C.c_int32),
                ("height", C.c_int32)]


# numpy dtypes matching the record structs
def record_dtypes():
    import numpy as np
    fill = np.dtype([("from_x", "<u2"), ("from_y", "<u2"), ("to_x", "<u2"), ("to_y", "<u2"),
                     ("emission_index", "<u4")])
    tile = np.dtype([("tile_x", "<i2"), ("tile_y", "<i2"), ("alpha_tile_id", "<u4"), ("path_id", "<u4"),
                     ("color", "<u2"), ("ctrl", "u1"), ("backdrop", "i1")])
    clip = np.dtype([("dest_tile_id", "<u4"), ("dest_backdrop", "<i4"), ("src_tile_id", "<u4"),
                     ("src_backdrop", "<i4")])
    path = np.dtype([("first_contour", "<u4"), ("contour_count", "<u4"), ("paint", "u1", (4,)),
                     ("clip_path", "<i4"), ("fill_rule", "u1"), ("blend_mode", "u1"), ("overlay", "<u2")])
    rect = np.dtype([("x0", "<i4"), ("y0", "<i4"), ("x1", "<i4"), ("y1", "<i4")])
    return fill, tile, clip, path, rect


_SIGS = {
    "PFCUDAStrokeToFill": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDAStrokeInput), C.POINTER(PFCUDAStrokeOutput)]),
    "PFCUDADashOutlines": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDAStrokeInput), C.POINTER(PFCUDADashInput),
                                       C.POINTER(PFCUDAOutlineOutput)]),
    "PFCUDAStrokeToFillDashed": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDAStrokeInput), C.POINTER(PFCUDADashInput),
                                             C.POINTER(PFCUDAStrokeOutput)]),
    "PFCUDAGradientSample": (C.c_int32, [C.POINTER(PFCUDAGradient), C.c_float, C.POINTER(PFColorU)]),
    "PFCUDAGradientRamp": (C.c_int32, [C.POINTER(PFCUDAGradient), C.c_void_p]),
    "PFCUDARendererCreate": (C.c_int32, [C.c_int32, C.POINTER(PFCUDARendererOptions), C.POINTER(C.c_void_p)]),
    "PFCUDARendererDestroy": (C.c_int32, [C.c_void_p]),
    "PFCUDARendererSetStream": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "PFCUDARendererSetOptions": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDARendererOptions)]),
    "PFCUDASceneUpload": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDASceneDesc)]),
    "PFCUDARenderScene": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_int32, C.c_int32,
                                      C.c_void_p, C.c_int32]),
    "PFCUDARenderSceneAsync": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_int32, C.c_int32,
                                           C.c_void_p]),
    "PFCUDARenderStatus": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "PFCUDARenderCoverage": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_int32, C.c_int32,
                                         C.c_void_p, C.c_int32]),
    "PFCUDAReadMasks": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64]),
    "PFCUDAReadRecords": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64,
                                      C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p, C.c_uint64]),
    "PFCUDAGetStats": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDARenderStats)]),
    "PFCUDASceneUploadBatch": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]),
    "PFCUDARenderBatch": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_uint32, C.c_uint32, C.c_int32,
                                      C.c_void_p]),
    "PFCUDARenderBatchAsync": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_uint32, C.c_uint32,
                                           C.c_int32, C.c_void_p]),
    "PFCUDAGraphCapture": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_uint32, C.c_uint32, C.c_int32,
                                       C.c_void_p]),
    "PFCUDAGraphLaunch": (C.c_int32, [C.c_void_p]),
    "PFCUDAGraphRelease": (C.c_int32, [C.c_void_p]),
    "PFCUDASetTuning": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDATuning)]),
    "PFCUDAGetTuning": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDATuning)]),
    "PFCUDAAutotune": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_uint32, C.c_uint32, C.c_int32,
                                   C.c_void_p, C.c_int32, C.POINTER(PFCUDATuning)]),
    "PFCUDASetProfiling": (C.c_int32, [C.c_void_p, C.c_int32]),
    "PFCUDAGetStageTimes": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32]),
    "PFCUDAExclusiveScan": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]),
    "PFCUDAExclusiveScanNoAlloc": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "PFCUDASetPoints": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_int32]),
    "PFCUDARenderDiff": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_uint32, C.c_uint32, C.c_int32,
                                     C.c_int32, C.c_void_p, C.c_void_p]),
    "PFCUDARenderDiffAsync": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDABuildOptions), C.c_uint32, C.c_uint32,
                                          C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]),
    "PFCUDABackward": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "PFCUDAStatusString": (C.c_char_p, [C.c_int32]),
    "PFCUDAPipelineCreate": (C.c_int32, [C.c_int32, C.c_int32, C.POINTER(PFCUDARendererOptions),
                                         C.POINTER(C.c_void_p)]),
    "PFCUDAPipelineDestroy": (C.c_int32, [C.c_void_p]),
    "PFCUDAPipelineSubmit": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDASceneDesc), C.POINTER(PFCUDABuildOptions),
                                         C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.POINTER(C.c_uint64)]),
    "PFCUDAPipelinePoll": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(C.c_int32)]),
    "PFCUDAPipelineWait": (C.c_int32, [C.c_void_p, C.c_uint64]),
}

# The seeded scene generators (include/pathfinder_cuda_scenes.h) live in their
# own host-only library, libpfscenes.so: generating a test or benchmark scene
# does not load the renderer.
SCENES_LIB_PATH = os.path.join(HERE, "libpfscenes.so")
_SCENE_SIGS = {
    "PFCUDASceneGenerate": (C.c_int32, [C.POINTER(PFCUDASceneParams), C.POINTER(C.c_void_p)]),
    "PFCUDASceneGetDesc": (C.c_int32, [C.c_void_p, C.POINTER(PFCUDASceneDesc), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int32)]),
    "PFCUDASceneGetCells": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "PFCUDASceneDestroy": (C.c_int32, [C.c_void_p]),
}


def bind_scene_generator(l: C.CDLL) -> C.CDLL:
    """Declare the scene generator's signatures on a library that exports them."""
    for name, (res, args) in _SCENE_SIGS.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args
    return l


_scenes_lib = None


def scenes_lib() -> C.CDLL:
    """The loaded scene generator library (raises if it is missing)."""
    global _scenes_lib
    if _scenes_lib is None:
        if not os.path.exists(SCENES_LIB_PATH):
            raise ImportError(f"{SCENES_LIB_PATH} is missing: run pathfinder_gb300.build.build()")
        _scenes_lib = bind_scene_generator(C.CDLL(SCENES_LIB_PATH))
    return _scenes_lib

_lib = None


def lib() -> C.CDLL:
    """The loaded CUDA renderer library (raises if it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run pathfinder_gb300.build.build() "
                              "(there is no CPU fallback)")
        l = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


class PFCUDAError(RuntimeError):
    def __init__(self, code: int, what: str):
        msg = lib().PFCUDAStatusString(code).decode()
        super().__init__(f"{what}: {msg} (status {code})")
        self.code = code


def check(code: int, what: str) -> None:
    if code != PF_CUDA_OK:
        raise PFCUDAError(code, what)
