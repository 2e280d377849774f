"""Differentiable rendering over the C ABI: PFCUDASetPoints, PFCUDARenderDiff
and PFCUDABackward behind a thin ``torch.autograd.Function``.

It is used by the gradient checks and the fitting harness only; all
arithmetic of the forward and of the adjoint runs in the library's kernels.
The reference has no backward pass.
"""
from __future__ import annotations

import numpy as np
import torch

from .batch import SceneBatch
from .renderer import BuildOptions, Renderer
from .scene import Scene

_LEGACY_STREAM = 1  # cudaStreamLegacy: torch's default stream reports handle 0


def _bind_stream(r: Renderer) -> None:
    h = torch.cuda.current_stream().cuda_stream
    r.set_stream(h if h else _LEGACY_STREAM)


class DiffRenderer:
    """A renderer holding one scene or a batch of scenes for differentiable
    frames: ``image = dr(points, alpha)`` with ``points`` [N, 2] (every point
    of the scene or batch, batch order) and ``alpha`` one paint alpha per draw
    path, both float32 CUDA tensors.  A single scene renders into a
    height x width image; a batch into its targets (``SceneBatch.packed``:
    one flat buffer of ``total_pixels``)."""

    def __init__(self, scenes: Scene | SceneBatch, device: int = 0, options: BuildOptions | None = None,
                 renderer: Renderer | None = None, sync: bool = True):
        self.renderer = renderer or Renderer(device)
        self.options = options
        # sync=False enqueues frames after the first without a status readback
        # (check renderer.render_status() at the end of a run)
        self.sync = sync
        self.device = torch.device("cuda", device)
        if isinstance(scenes, SceneBatch):
            self.batch = scenes
            self.renderer.upload_batch(scenes)
            self.count = len(scenes)
            self.width = self.height = 0
            self.shape = (int(scenes.total_pixels),)
            all_scenes = scenes.scenes
        else:
            self.batch = None
            self.renderer.upload_scene(scenes)
            self.count = 1
            self.width, self.height = scenes.width, scenes.height
            self.shape = (scenes.height, scenes.width)
            all_scenes = [scenes]
        self.points0 = torch.from_numpy(np.concatenate([np.asarray(s.points, np.float32).reshape(-1, 2)
                                                        for s in all_scenes])).to(self.device)
        self.alpha0 = torch.from_numpy(np.concatenate([s.draw_paths["paint"][:, 3].astype(np.float32) / 255.0
                                                       for s in all_scenes])).to(self.device)
        self.n_points = int(self.points0.shape[0])
        self.n_draw = int(self.alpha0.shape[0])
        self._epoch = 0

    def __call__(self, points: torch.Tensor, alpha: torch.Tensor | None = None) -> torch.Tensor:
        if alpha is None:
            alpha = self.alpha0
        return _RenderDiff.apply(points, alpha, self)

    # plain calls, without autograd
    def forward(self, points: torch.Tensor, alpha: torch.Tensor) -> torch.Tensor:
        r = self.renderer
        _bind_stream(r)
        r.set_points(points.detach().to(torch.float32).contiguous())
        out = torch.zeros(self.shape, dtype=torch.float32, device=self.device)
        r.render_diff(out, 0, self.count, self.width, self.height, alpha.detach().to(torch.float32).contiguous(),
                      self.options, sync=self.sync or self._epoch == 0)
        self._epoch += 1
        return out

    def backward(self, d_image: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        r = self.renderer
        _bind_stream(r)
        gp = torch.empty((self.n_points, 2), dtype=torch.float32, device=self.device)
        ga = torch.empty((self.n_draw,), dtype=torch.float32, device=self.device)
        r.backward(d_image.detach().to(torch.float32).contiguous(), gp, ga)
        return gp, ga


class _RenderDiff(torch.autograd.Function):
    @staticmethod
    def forward(ctx, points, alpha, dr: DiffRenderer):
        out = dr.forward(points, alpha)
        ctx.dr = dr
        ctx.epoch = dr._epoch
        return out

    @staticmethod
    def backward(ctx, grad):
        dr = ctx.dr
        if dr._epoch != ctx.epoch:
            raise RuntimeError("the adjoint needs the renderer's latest differentiable frame")
        gp, ga = dr.backward(grad)
        return gp, ga, None


def render_coverage(dr: DiffRenderer, points: torch.Tensor, alpha: torch.Tensor | None = None) -> torch.Tensor:
    """Differentiable single-channel FP32 coverage of the renderer's scene(s)."""
    return dr(points, alpha)
