"""The CUDA differentiable frame and its adjoint against the FP64 oracle:
image within 5e-4, gradients to control points and paint alphas within 1e-3
relative (max norm and L2) for the same dL/dimage."""
import numpy as np
import pytest

import oracle
import pathfinder_gb300 as pf
from diffscenes import blobs, mixed

pytestmark = pytest.mark.gpu

IMG_TOL = 5e-4
GRAD_TOL = 1e-3


def _rel_err(got, ref):
    got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
    scale = max(np.abs(ref).max(), 1e-30)
    return np.abs(got - ref).max() / scale, np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)


def _compare(scene, W, H, options=None, seed=1, target=None):
    torch = pytest.importorskip("torch")
    from pathfinder_gb300.diff import DiffRenderer
    ora = oracle.DiffOracle(scene, W, H, options)
    if target is None:
        rng = np.random.default_rng(seed)
        target = ora.render(ora.points + rng.normal(0, 2.0, ora.points.shape))
    ref = ora.render()
    dr = DiffRenderer(scene, options=options)
    img = dr.forward(dr.points0, dr.alpha0).cpu().numpy()
    assert np.abs(img - ref).max() <= IMG_TOL, f"image differs by {np.abs(img - ref).max()}"
    g = 2.0 * (ref - target)
    gp, ga = dr.backward(torch.from_numpy(g.astype(np.float32)).cuda())
    torch.cuda.synchronize()
    gp_o, ga_o = ora.grad(g.astype(np.float32).astype(np.float64))
    e_max, e_l2 = _rel_err(gp.cpu().numpy(), gp_o)
    assert e_max <= GRAD_TOL and e_l2 <= GRAD_TOL, f"dL/dpoints: max rel {e_max:.2e}, L2 rel {e_l2:.2e}"
    a_max, a_l2 = _rel_err(ga.cpu().numpy(), ga_o)
    assert a_max <= GRAD_TOL and a_l2 <= GRAD_TOL, f"dL/dalpha: max rel {a_max:.2e}, L2 rel {a_l2:.2e}"
    return dr, gp_o


def test_cubic_1k_gradients_match_fp64_oracle(built):
    """256 closed cubic paths, 4,096 control points, 1024^2 FP32 coverage,
    L2 loss against the render of the points + N(0, 2 px)."""
    s = pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=1)
    t = pf.generate_scene(pf.PF_SCENE_CUBIC_1K, seed=1, jitter_sigma=2.0, jitter_seed=2)
    target = oracle.DiffOracle(t, 1024, 1024).render()
    _compare(s, 1024, 1024, target=target)


@pytest.mark.parametrize("kind", ["edge", "even_odd_holes", "holes", "mixed_clip"])
def test_small_scene_gradients_match_oracle(built, kind):
    if kind == "edge":
        s = blobs(W=96, H=96, n=6, seed=3, edge=True)
    elif kind == "even_odd_holes":
        s = blobs(W=96, H=96, n=4, seed=5, even_odd=True, holes=True)
    elif kind == "holes":
        s = blobs(W=96, H=96, n=4, seed=6, holes=True)
    else:
        s = mixed(W=96, H=96, n=5, seed=2)
    _compare(s, 96, 96)


def test_transformed_scene_gradients_match_oracle(built):
    s = blobs(W=96, H=96, n=4, seed=8)
    _compare(s, 96, 96, options=pf.BuildOptions(pf.Transform2F(0.8, -0.3, 0.25, 0.9, 12.0, 6.0)))


def test_stars_gradients_match_oracle(built):
    """Quadratic and cubic stars (512^2): the quadratic chain through the
    degree elevation."""
    s = pf.generate_scene(pf.PF_SCENE_STARS_512, seed=4)
    _compare(s, 512, 512)


def test_autograd_function_matches_explicit_adjoint(built):
    torch = pytest.importorskip("torch")
    from pathfinder_gb300.diff import DiffRenderer
    s = blobs(W=128, H=128, n=6, seed=12)
    dr = DiffRenderer(s)
    target = torch.rand((128, 128), device="cuda")
    pts = dr.points0.clone().requires_grad_(True)
    alpha = dr.alpha0.clone().requires_grad_(True)
    loss = ((dr(pts, alpha) - target) ** 2).sum()
    loss.backward()
    img = dr.forward(dr.points0, dr.alpha0)
    gp, ga = dr.backward(2.0 * (img - target))
    assert torch.allclose(pts.grad, gp, rtol=1e-5, atol=1e-6)
    assert torch.allclose(alpha.grad, ga, rtol=1e-5, atol=1e-6)


def test_batch_gradients_equal_single_scene_gradients(built):
    """A packed batch of uneven scenes: one frame and one adjoint give each
    scene's own image and gradients."""
    torch = pytest.importorskip("torch")
    from pathfinder_gb300.diff import DiffRenderer
    scenes = [blobs(W=w, H=w, n=n, seed=20 + i) for i, (w, n) in enumerate([(64, 3), (128, 7), (96, 5)])]
    batch = pf.SceneBatch.packed(scenes)
    dr = DiffRenderer(batch)
    img = dr.forward(dr.points0, dr.alpha0)
    g = torch.rand_like(img)
    gp, ga = dr.backward(g)
    p0 = a0 = 0
    for s, off in zip(scenes, batch.offsets):
        n_px = s.width * s.height
        single = DiffRenderer(s)
        simg = single.forward(single.points0, single.alpha0)
        assert torch.allclose(img[off:off + n_px].view(s.height, s.width), simg, atol=1e-6)
        sgp, sga = single.backward(g[off:off + n_px].view(s.height, s.width))
        n_p, n_a = single.n_points, single.n_draw
        assert torch.allclose(gp[p0:p0 + n_p], sgp, rtol=1e-4, atol=1e-5)
        assert torch.allclose(ga[a0:a0 + n_a], sga, rtol=1e-4, atol=1e-5)
        p0 += n_p
        a0 += n_a


def test_backward_needs_the_latest_differentiable_frame(built):
    torch = pytest.importorskip("torch")
    from pathfinder_gb300.diff import DiffRenderer
    from pathfinder_gb300._abi import PFCUDAError
    s = blobs(W=64, H=64, n=2, seed=30)
    dr = DiffRenderer(s)
    img = dr.forward(dr.points0, dr.alpha0)
    dr.renderer.render_coverage(s, out=torch.zeros((64, 64), device="cuda"))  # a plain frame in between
    with pytest.raises(PFCUDAError):
        dr.backward(torch.ones_like(img))
