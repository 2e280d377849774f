"""Frames in flight: a stream of scenes rendered by several renderers at once,
each on its own CUDA stream and worker thread, so that one frame's upload and
image copy overlap the kernels of the others.

This is the host mirror of PFCUDAPipeline (include/pathfinder_cuda.h), the
CUDA level's counterpart of SceneProxy
(renderer/src/concurrent/scene_proxy.rs:11-20, :86-121).  SceneProxy builds
scenes on a worker thread and keeps a bounded number of render commands in
flight; here every stage of a frame is GPU work, so what is kept in flight is
whole frames, at most `depth` of them.  The workers are native threads of the
library: submitting returns at once, and waiting for a frame releases the
interpreter.
"""
from __future__ import annotations

import ctypes as C

from . import _abi
from .renderer import BuildOptions, RendererOptions, _ptr


class Frame:
    """One submitted frame: ``result()`` waits for it and returns its output
    buffer (raising the frame's error), ``done()`` asks without waiting."""

    def __init__(self, pipeline: "RenderPipeline", ticket: int, out):
        self._pipeline = pipeline
        self.ticket = ticket
        self._out = out
        self._code = None

    def done(self) -> bool:
        if self._code is not None:
            return True
        flag = C.c_int32()
        _abi.check(self._pipeline._lib.PFCUDAPipelinePoll(self._pipeline._h, self.ticket, C.byref(flag)),
                   "PFCUDAPipelinePoll")
        return bool(flag.value)

    def result(self):
        if self._code is None:
            self._code = self._pipeline._wait(self.ticket)
        _abi.check(self._code, "pipelined frame")
        return self._out


class RenderPipeline:
    """`depth` renderers on one device behind the library's worker threads.

    ``submit(scene, out)`` uploads the scene to the next free renderer and
    renders it (premultiplied RGBA8) into ``out``, a host numpy array or a
    CUDA tensor; the returned Frame's ``result()`` is ``out`` once written.
    With ``copy_image`` (the default) a host ``out`` is written by one
    device-to-host copy after the composite (PF_MEMORY_HOST_COPY), which the
    copy engine makes while the SMs run the other frames; use page-locked
    memory for it.  The scene and ``out`` are kept alive until their frame
    is waited for or the pipeline is closed; do not change them before.
    """

    def __init__(self, device: int = 0, depth: int = 3, options: RendererOptions | None = None,
                 copy_image: bool = True):
        self._lib = _abi.lib()
        self.depth = depth
        self.copy_image = copy_image
        self._h = C.c_void_p()
        self._held = {}  # ticket -> what the frame reads or writes
        o = (options or RendererOptions()).to_c()
        _abi.check(self._lib.PFCUDAPipelineCreate(device, depth, C.byref(o), C.byref(self._h)),
                   "PFCUDAPipelineCreate")

    def submit(self, scene, out, options: BuildOptions | None = None, width: int | None = None,
               height: int | None = None) -> Frame:
        if not self._h:
            raise RuntimeError("pipeline is closed")
        w, h = width or scene.width, height or scene.height
        p, mem = _ptr(out)
        if self.copy_image and mem == _abi.PF_MEMORY_HOST:
            mem = _abi.PF_MEMORY_HOST_COPY
        desc = scene.desc()
        bo = (options or BuildOptions()).to_c()
        ticket = C.c_uint64()
        _abi.check(self._lib.PFCUDAPipelineSubmit(self._h, C.byref(desc), C.byref(bo), w, h, C.c_void_p(p), mem,
                                                  C.byref(ticket)), "PFCUDAPipelineSubmit")
        self._held[ticket.value] = (scene, desc, bo, out)
        return Frame(self, ticket.value, out)

    def _wait(self, ticket: int) -> int:
        code = self._lib.PFCUDAPipelineWait(self._h, ticket)
        self._held.pop(ticket, None)
        return code

    def close(self) -> None:
        """Waits for every submitted frame and frees the renderers."""
        if self._h:
            self._lib.PFCUDAPipelineDestroy(self._h)
            self._h = C.c_void_p()
        self._held.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
