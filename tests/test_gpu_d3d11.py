"""The D3D11 level's tiling semantics on the CUDA level (uniform dicing into
1/256-px microlines, unclipped truncating bins) against the oracle's
restatement of the same mode: records bit-exact, coverage within 1/255,
images within 2/255."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from tests.parity import compare_images, compare_masks, compare_records

pytestmark = pytest.mark.gpu

CASES = [
    (pf.PF_SCENE_STARS_512, 1.0, 1),
    (pf.PF_SCENE_EDGE_CASES, 1.0, 1),
    (pf.PF_SCENE_SVG_4K, 0.02, 3),
    (pf.PF_SCENE_GLYPH_ATLAS, 0.02, 5),
    (pf.PF_SCENE_CUBIC_1K, 1.0, 11),
]


@pytest.fixture(scope="module")
def d3d11_renderer(built):
    r = pf.Renderer(0, pf.RendererOptions(d3d11_semantics=True))
    yield r
    r.close()


@pytest.mark.parametrize("workload,scale,seed", CASES)
def test_d3d11_semantics_parity(d3d11_renderer, workload, scale, seed):
    import oracle
    s = pf.generate_scene(workload, seed=seed, scale=scale)
    img = d3d11_renderer.render(s)
    fr = oracle.OracleFrame(s, d3d11=True)
    assert d3d11_renderer.stats().line_count == fr.line_count
    compare_records(s, d3d11_renderer.read_records(s), fr)
    compare_masks(d3d11_renderer, fr)
    ora, _ = fr.render(s.width, s.height)
    compare_images(img, ora)


def test_d3d11_semantics_with_transform(d3d11_renderer):
    import oracle
    s = pf.generate_scene(pf.PF_SCENE_STARS_512, seed=6)
    bo = pf.BuildOptions(pf.Transform2F(0.71, 0.52, -0.33, 0.88, 60.0, -20.5))
    img = d3d11_renderer.render(s, options=bo)
    fr = oracle.OracleFrame(s, bo, d3d11=True)
    compare_records(s, d3d11_renderer.read_records(s), fr)
    ora, _ = fr.render(s.width, s.height)
    compare_images(img, ora)


def test_d3d11_semantics_rejects_differentiable_frames(d3d11_renderer):
    torch = pytest.importorskip("torch")
    from pathfinder_gb300._abi import PFCUDAError
    s = pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=2, scale=0.05, width=128, height=128)
    d3d11_renderer.upload_scene(s)
    out = torch.zeros((128, 128), device="cuda")
    with pytest.raises(PFCUDAError):
        d3d11_renderer.render_diff(out, width=128, height=128)
