"""Known-answer cases for the tiler restatement, derived by hand from
renderer/src/tiler.rs:191-308 (DDA, auxiliary fills, backdrop steps),
renderer/src/builder.rs:509-616 (8.8 conversion, culls, backdrops) and
renderer/src/tiler.rs:93-163 (column prefix)."""
import numpy as np

import oracle
from tests.kat import poly_scene, rect_scene

INV = 0xFFFFFFFF


def fills_of(fr):
    f, t = fr.fills()
    tiles, _, _, _ = fr.tiles()
    out = []
    for i in range(len(f)):
        tt = tiles[t[i]]
        out.append(((int(tt["tile_x"]), int(tt["tile_y"])),
                    (int(f["from_x"][i]), int(f["from_y"][i]), int(f["to_x"][i]), int(f["to_y"][i]))))
    return out


def tile_map(fr):
    tiles, _, _, _ = fr.tiles()
    return {(int(t["tile_x"]), int(t["tile_y"])): (int(t["alpha_tile_id"]), int(t["backdrop"])) for t in tiles}


def test_tile_aligned_square():
    # [16,32]^2: one fill along the top edge; x clamps to 4095 (builder.rs:527-529)
    fr = oracle.OracleFrame(rect_scene(16, 16, 32, 32))
    assert fills_of(fr) == [((1, 1), (0, 0, 4095, 0))]
    assert tile_map(fr) == {(1, 1): (0, 0)}
    raw, cov = fr.masks()
    expect = np.full((16, 16), -1.0)
    expect[:, 15] = -(4095 / 256 - 15)
    assert np.allclose(raw[0], expect, atol=1e-12)


def test_rect_spanning_nine_tiles():
    fr = oracle.OracleFrame(rect_scene(8, 8, 40, 40))
    assert fills_of(fr) == [
        ((0, 0), (2048, 2048, 4095, 2048)),
        ((1, 0), (0, 2048, 4095, 2048)),
        ((2, 0), (0, 2048, 2048, 2048)),
        ((2, 1), (0, 0, 2048, 0)),          # enters through the top boundary (aux)
        ((2, 2), (0, 0, 2048, 0)),          # aux
        ((2, 2), (2048, 2048, 0, 2048)),
        ((1, 2), (4095, 2048, 0, 2048)),
        ((0, 2), (4095, 2048, 2048, 2048)),
        ((0, 2), (2048, 0, 0, 0)),          # leaves through the top boundary (aux)
        ((0, 1), (2048, 0, 0, 0)),          # aux
    ]
    assert tile_map(fr) == {
        (0, 0): (0, 0), (1, 0): (1, 0), (2, 0): (2, 0),
        (0, 1): (3, -1), (1, 1): (INV, -1), (2, 1): (4, 0),
        (0, 2): (5, -1), (1, 2): (6, -1), (2, 2): (7, 0),
    }
    _, cov = fr.masks()
    tiles, _, _, _ = fr.tiles()
    idx = {(int(t["tile_x"]), int(t["tile_y"])): i for i, t in enumerate(tiles)}
    assert np.all(cov[idx[(1, 1)]] == 1.0)             # solid interior
    left = cov[idx[(0, 1)]]
    assert np.allclose(left[:, :8], 0.0) and np.allclose(left[:, 8:], 1.0)


def test_corner_crossing_tie_breaks_to_x():
    # (8,8)->(24,24) meets the tile corner (16,16): t_max.x == t_max.y, step in x
    # first (tiler.rs:229-248); the zero-length piece in tile (1,0) is culled.
    fr = oracle.OracleFrame(poly_scene([(8, 8), (24, 24), (8, 24)]))
    assert fills_of(fr) == [
        ((0, 0), (2048, 2048, 4095, 4095)),
        ((1, 1), (0, 0, 2048, 2048)),
        ((1, 1), (2048, 2048, 0, 2048)),
        ((0, 1), (4095, 2048, 2048, 2048)),
        ((0, 1), (2048, 0, 0, 0)),
    ]
    assert tile_map(fr) == {(0, 0): (0, 0), (1, 0): (INV, 0), (0, 1): (1, -1), (1, 1): (2, 0)}


def test_vertical_edges_emit_cancelling_top_boundary_fills():
    # A zero-area path down and back up x = 10.  The vertical pieces are culled
    # (from_x == to_x, builder.rs:532-536) but each crossing of a tile's top
    # edge adds an auxiliary fill along that edge (tiler.rs:265-275): entering
    # on the way down, leaving on the way up.  The pairs cancel.
    fr = oracle.OracleFrame(poly_scene([(10, 5), (10, 50)]))
    assert fills_of(fr) == [
        ((0, 1), (0, 0, 2560, 0)), ((0, 2), (0, 0, 2560, 0)), ((0, 3), (0, 0, 2560, 0)),
        ((0, 3), (2560, 0, 0, 0)), ((0, 2), (2560, 0, 0, 0)), ((0, 1), (2560, 0, 0, 0)),
    ]
    raw, cov = fr.masks()
    assert np.all(raw == 0.0) and np.all(cov == 0.0)


def test_path_above_view_box_feeds_column_backdrops():
    # The part above the view box only moves backdrops of the column above the
    # tile rect (builder.rs:609-612); the rect starts at row 0.
    fr = oracle.OracleFrame(rect_scene(8, -40, 40, 24))
    tm = tile_map(fr)
    assert min(y for _, y in tm) == 0
    # interior tile (1,0): the top edge lies above the view box, so its winding
    # reaches it only through the above-rect column backdrop
    assert tm[(1, 0)] == (INV, -1)
