"""RenderPipeline's host logic with stand-in renderers (no GPU): at most
`depth` frames at once, each renderer used by one thread at a time, uploads
only when a renderer does not hold the scene, errors raised by the frame's
future, renderers closed with the pipeline."""
import threading
import time

import pytest

from pathfinder_gb300.pipeline import RenderPipeline


class FakeScene:
    def __init__(self, sid):
        self.id, self.epoch = sid, 0


class FakeRenderer:
    lock = threading.Lock()
    running = 0
    peak = 0

    def __init__(self):
        self.busy = False
        self.held = None
        self.uploads = 0
        self.closed = False

    def upload_scene(self, scene, force=False):
        assert not self.busy, "renderer used by two threads at once"
        if force or self.held != (scene.id, scene.epoch):
            self.uploads += 1
            self.held = (scene.id, scene.epoch)

    def render(self, scene, options=None, out=None, copy_image=False):
        assert not self.busy, "renderer used by two threads at once"
        self.busy = True
        with FakeRenderer.lock:
            FakeRenderer.running += 1
            FakeRenderer.peak = max(FakeRenderer.peak, FakeRenderer.running)
        try:
            if scene.id < 0:
                raise RuntimeError("frame failed")
            time.sleep(0.01)
            out.append(scene.id)
            return out
        finally:
            with FakeRenderer.lock:
                FakeRenderer.running -= 1
            self.busy = False

    def close(self):
        self.closed = True


@pytest.fixture(autouse=True)
def _reset():
    FakeRenderer.running = FakeRenderer.peak = 0


@pytest.mark.parametrize("depth", [1, 2, 3])
def test_frames_in_flight_bounded_by_depth(depth):
    made = []

    def factory():
        made.append(FakeRenderer())
        return made[-1]

    with RenderPipeline(depth=depth, renderer_factory=factory) as p:
        outs = [[] for _ in range(12)]
        futs = [p.submit(FakeScene(i % 4), outs[i]) for i in range(12)]
        assert [f.result() for f in futs] == [[i % 4] for i in range(12)]
        assert len(p.renderers) == depth
    assert len(made) == depth and all(r.closed for r in made)
    assert FakeRenderer.peak == depth


def test_upload_only_when_the_renderer_lacks_the_scene():
    r = FakeRenderer()
    with RenderPipeline(depth=1, renderer_factory=lambda: r) as p:
        s = FakeScene(7)
        for _ in range(5):
            p.submit(s, []).result()
        assert r.uploads == 1
        p.submit(s, [], force=True).result()
        assert r.uploads == 2


def test_errors_surface_through_the_future():
    with RenderPipeline(depth=2, renderer_factory=FakeRenderer) as p:
        bad = p.submit(FakeScene(-1), [])
        good = p.submit(FakeScene(3), [])
        with pytest.raises(RuntimeError, match="frame failed"):
            bad.result()
        assert good.result() == [3]
        # the failed frame returned its renderer: later frames still run
        assert [p.submit(FakeScene(k), []).result() for k in range(4)] == [[0], [1], [2], [3]]


def test_closed_pipeline_refuses_work_and_bad_depth():
    p = RenderPipeline(depth=1, renderer_factory=FakeRenderer)
    p.close()
    with pytest.raises(RuntimeError):
        p.submit(FakeScene(0), [])
    with pytest.raises(ValueError):
        RenderPipeline(depth=0, renderer_factory=FakeRenderer)


def test_failed_construction_closes_what_was_made():
    made = []

    def factory():
        if len(made) == 2:
            raise RuntimeError("no device")
        made.append(FakeRenderer())
        return made[-1]

    with pytest.raises(RuntimeError, match="no device"):
        RenderPipeline(depth=3, renderer_factory=factory)
    assert len(made) == 2 and all(r.closed for r in made)
