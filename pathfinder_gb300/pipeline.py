"""Frames in flight: a stream of scenes rendered by several renderers at once,
each on its own CUDA stream and host thread, so that one frame's upload and
image write-back overlap the kernels of another.

This is the CUDA level's counterpart of SceneProxy
(renderer/src/concurrent/scene_proxy.rs:11-20, :86-121).  SceneProxy moves
scene building off the thread that drives the GPU and keeps a bounded number
of render commands in flight.  Here every stage of a frame is GPU work, so
what overlaps is whole frames, at most `depth` of them.  Each renderer is used
by one thread at a time (renderers are not thread-safe, as the reference's
`&mut Renderer` is not), and the C ABI selects each renderer's device for the
duration of every call.
"""
from __future__ import annotations

import queue
from concurrent.futures import Future, ThreadPoolExecutor

from .renderer import BuildOptions, Renderer, RendererOptions


class RenderPipeline:
    """`depth` renderers on one device behind a pool of `depth` host threads.

    ``submit(scene, out)`` uploads the scene to the next free renderer (when
    that renderer does not hold it yet, or always with ``force``) and renders
    it into ``out``; the returned future's result is ``out`` once the frame is
    written.  With ``copy_image`` (the default) a host ``out`` is written by a
    device-to-host copy after each composite, which the copy engine makes
    while the SMs run the other frames in flight.  A frame writes only its
    own ``out``: do not reuse that buffer before its future is done.  Errors
    of a frame are raised by its future.
    """

    def __init__(self, device: int = 0, depth: int = 3, options: RendererOptions | None = None,
                 renderer_factory=None, copy_image: bool = True):
        if depth < 1:
            raise ValueError("depth must be at least 1")
        self.copy_image = copy_image
        make = renderer_factory or (lambda: Renderer(device, options))
        self.depth = depth
        self._renderers = []
        try:
            for _ in range(depth):
                self._renderers.append(make())
        except Exception:
            for r in self._renderers:
                r.close()
            raise
        self._free: queue.SimpleQueue = queue.SimpleQueue()
        for r in self._renderers:
            self._free.put(r)
        self._pool = ThreadPoolExecutor(max_workers=depth, thread_name_prefix="pf-frame")

    @property
    def renderers(self) -> list:
        return list(self._renderers)

    def _frame(self, scene, out, options, force):
        # a task starts only on one of `depth` workers, so a renderer is free
        r = self._free.get()
        try:
            r.upload_scene(scene, force=force)
            return r.render(scene, options, out=out, copy_image=self.copy_image)
        finally:
            self._free.put(r)

    def submit(self, scene, out, options: BuildOptions | None = None, force: bool = False) -> Future:
        if self._pool is None:
            raise RuntimeError("pipeline is closed")
        return self._pool.submit(self._frame, scene, out, options, force)

    def close(self) -> None:
        if self._pool is not None:
            self._pool.shutdown(wait=True)
            self._pool = None
        for r in self._renderers:
            r.close()
        self._renderers = []

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
