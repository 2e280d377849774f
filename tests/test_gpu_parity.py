"""CUDA level vs the oracle: bit-exact records, coverage within 1/255,
images within 2/255 — on seeded scenes small enough for the oracle."""
import numpy as np
import pytest

import pathfinder_gb300 as pf
from tests.parity import compare_images, compare_masks, compare_records

pytestmark = pytest.mark.gpu

CASES = [
    (pf.PF_SCENE_STARS_512, 1.0, 1),
    (pf.PF_SCENE_STARS_512, 1.0, 7),
    (pf.PF_SCENE_EDGE_CASES, 1.0, 1),
    (pf.PF_SCENE_SVG_4K, 0.02, 3),
    (pf.PF_SCENE_GLYPH_ATLAS, 0.02, 5),
    (pf.PF_SCENE_CUBIC_1K, 1.0, 11),
]


@pytest.mark.parametrize("workload,scale,seed", CASES)
def test_records_masks_image(renderer, workload, scale, seed):
    import oracle
    s = pf.generate_scene(workload, seed=seed, scale=scale)
    img = renderer.render(s)
    fr = oracle.OracleFrame(s)
    rec = renderer.read_records(s)
    compare_records(s, rec, fr)
    compare_masks(renderer, fr)
    ora, _ = fr.render(s.width, s.height)
    compare_images(img, ora)
