"""SVG documents through the front-end with strokes converted on the GPU:
the scene equals the one built with the oracle's stroker (bit for bit) and the
GPU frame matches the oracle frame."""
import numpy as np
import pytest

from pathfinder_gb300.svg import load_svg
from tests import svgdocs
from tests.parity import compare_images
from tests.test_svg import OracleStroker

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_svg_document_parity(renderer, seed):
    import oracle
    doc = svgdocs.document(seed, n=40)
    g = load_svg(doc, renderer).scene
    o = load_svg(doc, OracleStroker()).scene
    assert np.array_equal(g.points.view(np.uint32), o.points.view(np.uint32))
    assert np.array_equal(g.flags, o.flags) and np.array_equal(g.contour_starts, o.contour_starts)
    img = renderer.render(g)
    ora, _ = oracle.OracleFrame(o).render(o.width, o.height)
    compare_images(img, ora)
