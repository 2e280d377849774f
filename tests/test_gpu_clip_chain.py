"""Clip chains (a clip path clipped by another, the D3D11 level's clip
levels): records bit-exact, coverage within 1/255 and images within 2/255 of
the oracle; cycles are rejected."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from tests.parity import compare_images, compare_masks, compare_records

pytestmark = pytest.mark.gpu


def _blob(cx, cy, r, k, rng, quad=True):
    c = pf.Contour()
    ang = np.sort(rng.uniform(0, 2 * np.pi, k))
    pts = [(cx + r * rng.uniform(0.7, 1.0) * np.cos(a), cy + r * rng.uniform(0.7, 1.0) * np.sin(a)) for a in ang]
    c.push_endpoint(*pts[0])
    for i in range(1, k + 1):
        x, y = pts[i % k]
        if quad and i % 2:
            px, py = pts[i - 1]
            c.push_quadratic((px + x) / 2 + rng.normal(0, 4), (py + y) / 2 + rng.normal(0, 4), x, y)
        else:
            c.push_endpoint(x, y)
    c.close()
    return pf.Outline([c])


def chain_scene(seed=1, W=192, H=160):
    rng = np.random.default_rng(seed)
    s = pf.Scene()
    s.set_view_box(pf.RectF(0, 0, W, H))
    c0 = s.push_clip_path(pf.ClipPath(_blob(96, 80, 70, 12, rng)))
    c1 = s.push_clip_path(pf.ClipPath(_blob(110, 70, 55, 10, rng), clip_path=c0))
    c2 = s.push_clip_path(pf.ClipPath(_blob(80, 90, 50, 9, rng), pf.FillRule.EVEN_ODD, clip_path=c1))
    c3 = s.push_clip_path(pf.ClipPath(_blob(40, 40, 30, 8, rng)))  # an unclipped clip
    for clip, rule, a in [(c2, pf.FillRule.WINDING, 230), (c1, pf.FillRule.EVEN_ODD, 160), (c0, pf.FillRule.WINDING, 255),
                          (c3, pf.FillRule.WINDING, 200), (None, pf.FillRule.WINDING, 120), (c2, pf.FillRule.WINDING, 255)]:
        s.push_draw_path(pf.DrawPath(_blob(rng.uniform(50, 140), rng.uniform(40, 120), rng.uniform(30, 70), 11, rng),
                                     pf.ColorU(int(rng.integers(0, 256)), int(rng.integers(0, 256)), 90, a), rule,
                                     clip_path=clip))
    return s


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_clip_chain_parity(renderer, seed):
    import oracle
    s = chain_scene(seed)
    img = renderer.render(s)
    fr = oracle.OracleFrame(s)
    rec = renderer.read_records(s)
    compare_records(s, rec, fr)
    assert (rec["tiles"]["ctrl"] & 0x4).any(), "no tile behind a clip chain"
    compare_masks(renderer, fr)
    ora, _ = fr.render(s.width, s.height)
    compare_images(img, ora)


def test_clip_cycle_rejected(renderer):
    import oracle
    from pathfinder_gb300._abi import PFCUDAError
    s = chain_scene(4)
    s.clip_paths["clip_path"][0] = 2  # c0 <- c2 <- c1 <- c0
    s.epoch += 1
    with pytest.raises(PFCUDAError):
        renderer.render(s)
    with pytest.raises(ValueError):
        oracle.OracleFrame(s)
