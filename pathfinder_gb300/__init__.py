"""pathfinder_gb300 — Pathfinder's compute rasterization path as a CUDA
renderer level for one GB300 (sm_103a).

The package is the host-side mirror of the reference's Scene / Renderer API
over the C ABI in ``include/pathfinder_cuda.h``; all work runs in the
hand-written kernels of ``libpathfinder_cuda.so``.  There is no CPU fallback.
"""
from .scene import (ClipPath, ColorF, ColorU, Contour, DrawPath, FillRule, Outline, RectF, Scene,
                    generate_scene)
from .paint import BlendMode, ColorStop, Gradient, GradientKind, GradientWrap, Pattern, PatternFilterKind
from .stroke import LineCap, LineJoin, StrokeStyle
from .renderer import (BuildOptions, Renderer, RendererLevel, RendererOptions, RenderStats, Transform2F)
from . import _abi
from .batch import SceneBatch, target
from .pipeline import RenderPipeline

PF_CUDA_FORMAT_RGBA8 = _abi.PF_CUDA_FORMAT_RGBA8
PF_CUDA_FORMAT_R8 = _abi.PF_CUDA_FORMAT_R8
PF_CUDA_FORMAT_F32 = _abi.PF_CUDA_FORMAT_F32

PF_SCENE_STARS_512 = _abi.PF_SCENE_STARS_512
PF_SCENE_SVG_4K = _abi.PF_SCENE_SVG_4K
PF_SCENE_GLYPH_ATLAS = _abi.PF_SCENE_GLYPH_ATLAS
PF_SCENE_CUBIC_1K = _abi.PF_SCENE_CUBIC_1K
PF_SCENE_EDGE_CASES = _abi.PF_SCENE_EDGE_CASES

__all__ = [
    "ClipPath", "ColorF", "ColorU", "Contour", "DrawPath", "FillRule", "Outline", "RectF", "Scene",
    "generate_scene", "BuildOptions", "Renderer", "RendererLevel", "RendererOptions", "RenderStats",
    "Transform2F", "PF_SCENE_STARS_512", "PF_SCENE_SVG_4K", "PF_SCENE_GLYPH_ATLAS", "PF_SCENE_CUBIC_1K",
    "PF_SCENE_EDGE_CASES", "BlendMode", "ColorStop", "Gradient", "GradientKind", "GradientWrap", "Pattern", "PatternFilterKind", "LineCap",
    "LineJoin", "StrokeStyle", "SceneBatch", "RenderPipeline",
]
