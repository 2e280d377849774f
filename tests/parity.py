"""Helpers comparing the CUDA level's records and images with the oracle."""
import numpy as np

COVERAGE_TOL = 1.0 / 255.0   # per-pixel coverage vs the FP64 formula


def canonical_gpu_fills(rec):
    f, t = rec["fills"], rec["fill_tile"]
    order = np.argsort(f["emission_index"], kind="stable")
    return f[order], t[order]


def compare_records(scene, rec, fr):
    """Bit-exact comparison of fills (canonical order), tiles, clips and z-buffer."""
    of, oft = fr.fills()
    gf, gft = canonical_gpu_fills(rec)
    assert len(gf) == len(of), f"fill count {len(gf)} != oracle {len(of)}"
    assert np.array_equal(gf["emission_index"], np.arange(len(of), dtype=np.uint32)), "emission indices"
    for k in ("from_x", "from_y", "to_x", "to_y"):
        bad = np.nonzero(gf[k] != of[k])[0]
        assert len(bad) == 0, f"fill field {k} differs at {bad[:10]} gpu={gf[bad[:5]]} oracle={of[bad[:5]]}"
    assert np.array_equal(gft, oft), "fill tile assignment differs"
    tiles, clips, offs, rects = fr.tiles()
    assert np.array_equal(rec["path_tile_offsets"], offs), "path tile offsets"
    gr = rec["path_tile_rects"]
    for k in ("x0", "y0", "x1", "y1"):
        assert np.array_equal(gr[k], rects[k]), f"tile rect {k}"
    gt = rec["tiles"]
    assert len(gt) == len(tiles)
    for k in tiles.dtype.names:
        bad = np.nonzero(gt[k] != tiles[k])[0]
        assert len(bad) == 0, f"tile field {k} differs at {bad[:10]}: gpu={gt[bad[:5]]} oracle={tiles[bad[:5]]}"
    nclip = len(scene.clip_paths)
    first_draw = int(offs[nclip])
    for k in clips.dtype.names:
        assert np.array_equal(rec["clips"][k][first_draw:], clips[k][first_draw:]), f"clip field {k}"
    assert np.array_equal(rec["z_buffer"], fr.zbuffer()), "z-buffer"


def compare_masks(renderer, fr, tol=COVERAGE_TOL):
    ga, gt = renderer.read_masks()
    oa, ot = fr.masks()
    assert ga.shape == oa.shape and gt.shape == ot.shape
    ea = float(np.abs(ga - oa).max()) if ga.size else 0.0
    et = float(np.abs(gt - ot).max()) if gt.size else 0.0
    assert ea <= tol, f"raw mask error {ea * 255:.3f}/255"
    assert et <= tol, f"tile coverage error {et * 255:.3f}/255"
    return ea, et


def compare_images(gpu, ora, max_diff=2, frac_exact=0.99):
    d = np.abs(gpu.astype(np.int32) - ora.astype(np.int32))
    if d.max() > max_diff:
        dm = d.max(-1) if d.ndim == 3 else d
        ys, xs = np.nonzero(dm > max_diff)
        where = ", ".join(f"({y},{x}) gpu={gpu[y, x].tolist()} ora={ora[y, x].tolist()}" for y, x in zip(ys[:4], xs[:4]))
        raise AssertionError(f"image max diff {d.max()} at {len(ys)} pixels, x {xs.min()}..{xs.max()}, "
                             f"y {ys.min()}..{ys.max()}: {where}")
    exact = float((d == 0).mean())
    assert exact >= frac_exact, f"only {exact:.4f} of channels exact"
    return int(d.max()), exact
