"""Plain frames flatten in one pass: each block of the flattening kernel takes
its range of lines with one atomic, so the frame's line order depends on the
schedule.  Frames run for record read-back flatten in depth-first order (count,
scan, emit).  No output may depend on which: fill counts, raw masks (integer
sums of the same fills) and resolved tile coverage of a plain frame must equal
those of the ordered frame bit for bit."""
import numpy as np
import pytest

import pathfinder_gb300 as pf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("workload, seed, scale", [(pf.PF_SCENE_SVG_4K, 2, 0.05), (pf.PF_SCENE_CUBIC_1K, 3, 1.0),
                                                    (pf.PF_SCENE_EDGE_CASES, 1, 1.0)])
def test_plain_frame_equals_ordered_frame(renderer, workload, seed, scale):
    s = pf.generate_scene(workload, seed=seed, scale=scale)
    renderer.render(s)
    st_plain = renderer.stats()
    a_plain, t_plain = renderer.read_masks()  # from the plain frame's fills
    renderer.read_records(s)  # re-runs the frame with its lines in depth-first order
    st_ord = renderer.stats()
    a_ord, t_ord = renderer.read_masks()
    for k in ("line_count", "fill_count", "tile_count", "alpha_tile_count", "visible_tile_count"):
        assert getattr(st_plain, k) == getattr(st_ord, k), k
    assert st_plain.line_count > 0
    assert np.array_equal(a_plain, a_ord)
    assert np.array_equal(t_plain, t_ord)
