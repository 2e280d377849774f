"""The FP64 differentiable oracle against central finite differences
(h = 1e-3 px, FP64) with each curve's subdivision held fixed, and against the
FP64 parity oracle's image.  CPU only: these pin the checker of the CUDA
adjoint."""
import numpy as np
import pytest

import oracle
import pathfinder_gb300 as pf
from diffscenes import blobs, mixed

H_FD = 1e-3


def _loss_fn(d, target):
    def loss(points, alpha):
        img = d.render(points, alpha)
        return float(((img - target) ** 2).sum()), img
    return loss


def _check_fd(d, target, coords, tol=2e-4, build_alpha=True):
    """Analytic gradient vs central differences at `coords` ((point, axis)
    pairs).  Coordinates whose one-sided differences disagree sit on a
    coverage kink and are skipped (at most a quarter of them)."""
    loss = _loss_fn(d, target)
    p0, a0 = d.points.copy(), d.alpha.copy()
    L0, img = loss(p0, a0)
    gp, ga = d.grad(2.0 * (img - target))
    scale = max(np.abs(gp).max(), 1e-12)
    skipped = 0
    for i, c in coords:
        pp = p0.copy(); pp[i, c] += H_FD
        pm = p0.copy(); pm[i, c] -= H_FD
        Lp, Lm = loss(pp, a0)[0], loss(pm, a0)[0]
        right, left = (Lp - L0) / H_FD, (L0 - Lm) / H_FD
        if abs(right - left) > 0.05 * scale:
            skipped += 1
            continue
        fd = (Lp - Lm) / (2 * H_FD)
        assert abs(fd - gp[i, c]) <= tol * scale + 1e-9, f"point {i} axis {c}: fd {fd} analytic {gp[i, c]}"
    assert skipped <= len(coords) // 4
    if build_alpha:
        for k in range(min(4, d.draw_path_count)):
            ap = a0.copy(); ap[k] += H_FD
            am = a0.copy(); am[k] -= H_FD
            fd = (loss(p0, ap)[0] - loss(p0, am)[0]) / (2 * H_FD)
            assert abs(fd - ga[k]) <= 1e-6 * max(np.abs(ga).max(), 1.0), f"alpha {k}: fd {fd} analytic {ga[k]}"
    return gp, ga


def _sample(d, n, seed=0):
    rng = np.random.default_rng(seed)
    idx = rng.choice(d.point_count * 2, size=min(n, d.point_count * 2), replace=False)
    return [divmod(int(k), 2) for k in idx]


def _target(d, seed=1, sigma=2.0):
    rng = np.random.default_rng(seed)
    return d.render(d.points + rng.normal(0, sigma, d.points.shape))


@pytest.mark.parametrize("edge", [False, True])
def test_cubic_blobs_fd(built, edge):
    s = blobs(W=96, H=96, n=6, seed=3, edge=edge)
    d = oracle.DiffOracle(s, 96, 96)
    _check_fd(d, _target(d), _sample(d, 40))


def test_even_odd_with_holes_fd(built):
    s = blobs(W=96, H=96, n=4, seed=5, even_odd=True, holes=True)
    d = oracle.DiffOracle(s, 96, 96)
    _check_fd(d, _target(d), _sample(d, 40))


def test_nonzero_with_holes_fd(built):
    s = blobs(W=96, H=96, n=4, seed=6, holes=True)
    d = oracle.DiffOracle(s, 96, 96)
    _check_fd(d, _target(d), _sample(d, 40))


def test_lines_quads_cubics_and_clip_fd(built):
    s = mixed(W=96, H=96, n=5, seed=2)
    d = oracle.DiffOracle(s, 96, 96)
    assert d.clip_path_count == 1
    gp, _ = _check_fd(d, _target(d), _sample(d, 48))
    # the clip path's points receive gradient through the clipped draw path
    clip_pts = slice(int(s.contour_starts[0]), int(s.contour_starts[1]))
    assert np.abs(gp[clip_pts]).max() > 0


def test_transform_fd(built):
    s = blobs(W=96, H=96, n=4, seed=8)
    bo = pf.BuildOptions(pf.Transform2F(0.8, -0.3, 0.25, 0.9, 12.0, 6.0))
    d = oracle.DiffOracle(s, 96, 96, bo)
    _check_fd(d, _target(d), _sample(d, 32))


def test_cubic_1k_fd_sample(built):
    """The 256-path, 1024^2 differentiable workload: FD at sampled coordinates."""
    s = pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=1)
    t = pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=1, jitter_sigma=2.0, jitter_seed=2)
    d = oracle.DiffOracle(s, 1024, 1024)
    assert d.point_count == 4096 and d.draw_path_count == 256
    target = oracle.DiffOracle(t, 1024, 1024).render()
    _check_fd(d, target, _sample(d, 16, seed=4), build_alpha=False)


def test_diff_image_close_to_parity_oracle(built):
    """Without the 8.8 rounding the differentiable image stays within the
    fill quantisation of the parity path's FP64 image."""
    s = blobs(W=128, H=128, n=8, seed=9)
    d = oracle.DiffOracle(s, 128, 128)
    img = d.render()
    _, ref = oracle.OracleFrame(s).render(128, 128, channels=1)
    diff = np.abs(img - ref)
    assert diff.max() < 1.0 / 32
    assert diff.mean() < 2e-3


def test_translation_moves_image(built):
    """Shifting every point by whole pixels shifts the FP64 image exactly
    (the winding integral is translation-covariant)."""
    s = blobs(W=96, H=96, n=3, seed=11)
    d = oracle.DiffOracle(s, 96, 96)
    img = d.render()
    moved = d.render(d.points + np.array([5.0, 3.0]))
    assert np.allclose(moved[3:, 5:], img[:-3, :-5], atol=1e-9)
