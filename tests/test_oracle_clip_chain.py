"""The oracle's clip-chain semantics on the CPU: for nonzero paths, a draw
path behind a chain of clip paths has, per pixel, the minimum of the
coverages of the draw path and of every clip level rendered alone."""
import numpy as np

import oracle
import pathfinder_gb300 as pf
from test_gpu_clip_chain import _blob


def _alone(outline, W, H):
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    s.push_draw_path(pf.DrawPath(outline, pf.ColorU(255, 255, 255, 255)))
    _, f64 = oracle.OracleFrame(s).render(W, H, channels=1)
    return f64


def test_chain_is_minimum_of_levels(built):
    W, H = 160, 128
    for seed in (5, 6):
        rng = np.random.default_rng(seed)
        outlines = [_blob(80, 64, 60, 12, rng), _blob(90, 60, 45, 10, rng), _blob(70, 70, 40, 9, rng),
                    _blob(rng.uniform(60, 100), rng.uniform(50, 80), 50, 11, rng)]
        s = pf.Scene()
        s.set_view_box(pf.RectF(0, 0, W, H))
        c0 = s.push_clip_path(pf.ClipPath(outlines[0]))
        c1 = s.push_clip_path(pf.ClipPath(outlines[1], clip_path=c0))
        c2 = s.push_clip_path(pf.ClipPath(outlines[2], clip_path=c1))
        s.push_draw_path(pf.DrawPath(outlines[3], pf.ColorU(255, 255, 255, 255), clip_path=c2))
        _, chained = oracle.OracleFrame(s).render(W, H, channels=1)
        expect = np.minimum.reduce([_alone(o, W, H) for o in outlines])
        assert np.abs(chained - expect).max() < 1e-9
        assert chained.max() > 0.5  # the chain leaves something visible
