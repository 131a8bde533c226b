"""Adjoint of the converged solution (zs_ba_adjoint) against an FP64 reference
gradient and central finite differences of whole solves. Loss: sum over free
poses of ||log T_k - log T_k^target||^2 (se(3) log coordinates). Tolerance:
1e-5 relative."""

import numpy as np
import pytest

from conftest import rel_err
from gradcheck import harness as H
from zeroslam_gb300 import scenes

pytestmark = pytest.mark.gpu

ADJ_TOL = 1e-5
FD_STEP = 1e-6


def _small(seed=31, K=8, L=200):
    sc = scenes.arc_scene(K, L, seed=seed, min_obs=2, iterations=50, **scenes.ADJOINT_INIT_NOISE)
    sc.pose_fixed[1] = 1
    return sc


def _setup(sc):
    from zeroslam_gb300 import ba

    h = ba.BundleAdjuster(precision=ba.FP64)
    x = H.converge(h, sc)
    loss = H.PoseLogLoss(H.targets_for(sc), sc.pose_fixed)
    a = loss.grad_local(x[0])
    duv, dint, rep = h.adjoint(a, None)
    return h, x, loss, a, duv, dint, rep


def test_adjoint_matches_fp64_reference(zs_lib, oracle):
    sc = _small()
    h, x, loss, a, duv, dint, rep = _setup(sc)
    h.close()
    assert rep.rel_residual < 1e-10, rep.rel_residual
    ref_uv, ref_int = H.reference_gradient(oracle, sc, x, a, np.zeros((sc.L, 3)))
    assert rel_err(dint, ref_int) < ADJ_TOL
    assert rel_err(duv, ref_uv) < ADJ_TOL


def _fd_check(sc, n_pixels, seed):
    """Central differences (step FD_STEP) of whole re-converged solves: each
    intrinsic, then either n_pixels single pixel coordinates or, with
    n_pixels=None, the directional derivative along u = dL/duv / max|dL/duv|
    (every pixel moves by at most FD_STEP). A single pixel of a scene with
    ~1e5 observations moves L by ~1e-12 for that step, below the rounding
    level of re-converged solves, so that scene is checked along u."""
    h, x, loss, a, duv, dint, rep = _setup(sc)
    try:
        ad, fd = [], []
        for c in range(4):
            vals = []
            for sgn in (1.0, -1.0):
                intr = list(sc.intrinsics)
                intr[c] += sgn * FD_STEP
                vals.append(H.loss_at(h, sc, x, loss, intrinsics=intr))
            fd.append((vals[0] - vals[1]) / (2 * FD_STEP))
            ad.append(dint[c])
        if n_pixels is None:
            u = duv / np.abs(duv).max()
            vals = [H.loss_at(h, sc, x, loss, uv=sc.obs_uv + sgn * FD_STEP * u) for sgn in (1.0, -1.0)]
            fd.append((vals[0] - vals[1]) / (2 * FD_STEP))
            ad.append(float(np.sum(duv * u)))
        else:
            rng = np.random.default_rng(seed)
            for o in rng.choice(sc.M, n_pixels, replace=False):
                for k in range(2):
                    vals = []
                    for sgn in (1.0, -1.0):
                        uv = sc.obs_uv.copy()
                        uv[o, k] += sgn * FD_STEP
                        vals.append(H.loss_at(h, sc, x, loss, uv=uv))
                    fd.append((vals[0] - vals[1]) / (2 * FD_STEP))
                    ad.append(duv[o, k])
    finally:
        h.close()
    ad, fd = np.array(ad), np.array(fd)
    # intrinsics and pixels are compared on their own scales
    assert rel_err(ad[:4], fd[:4]) < ADJ_TOL, (ad[:4], fd[:4])
    assert rel_err(ad[4:], fd[4:]) < ADJ_TOL, (ad[4:], fd[4:])


def test_adjoint_matches_central_differences_small(zs_lib):
    _fd_check(_small(seed=32), n_pixels=6, seed=1)


def test_adjoint_matches_central_differences_50_keyframes(zs_lib):
    """The differentiable-BA scene: 50 keyframes, 10,000 landmarks, ~4.6e5 observations."""
    _fd_check(scenes.adjoint_scene(), n_pixels=None, seed=2)


def test_torch_autograd_function(zs_lib):
    torch = pytest.importorskip("torch")
    BAFunction = H.make_autograd_function()
    sc = _small(seed=33, K=5, L=40)
    from zeroslam_gb300 import ba

    with ba.BundleAdjuster(precision=ba.FP64) as h:
        x = H.converge(h, sc)
    warm = sc.copy()
    warm.poses, warm.landmarks = x[0].copy(), x[1].copy()
    uv = torch.tensor(sc.obs_uv, dtype=torch.float64, requires_grad=True)
    intr = torch.tensor(sc.intrinsics, dtype=torch.float64, requires_grad=True)

    def f(u, i):
        return BAFunction.apply(u, i, warm, 0)

    assert torch.autograd.gradcheck(f, (uv, intr), eps=FD_STEP, atol=1e-8, rtol=ADJ_TOL, fast_mode=True)
