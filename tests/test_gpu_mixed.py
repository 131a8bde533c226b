"""The mixed form's reduced solve: conjugate gradients on the exact Schur
operator of the FP32 Jacobian (zeroslam_gb300/csrc/ba_inverse.cu, k_pcg),
preconditioned by the FP32 factor of the FP32-formed Schur complement.

A walk is a long, ill-conditioned trajectory (the weakest eigenvalues of S are
~1e-8 of the largest, where H_pp and W H_pl^T cancel): there the FP32-formed S
alone gives steps that are off by O(1) in the weakest directions. The mixed
steps must follow the FP64 steps (the FP32 rounding of the Jacobian alone
separates them by ~1e-5), the final cost must agree with FP64 to 1e-6, the
solve must repeat bit for bit, and a step must succeed where the FP32
factorisation of the FP32-formed S fails but the exact S is positive definite
(the preconditioner's shifted retry)."""

import numpy as np
import pytest

from conftest import rel_err
from zeroslam_gb300 import scenes

pytestmark = pytest.mark.gpu

MIXED_COST_TOL = 1e-6
STEP_TOL = 1e-3  # J' = fl32(J) against J: measured 1e-5..3e-5 on walks


def _ba(precision, **kw):
    from zeroslam_gb300 import ba

    return ba.BundleAdjuster(precision=precision, **kw)


_WALK = {}


def _walk():
    if "sc" not in _WALK:
        _WALK["sc"] = scenes.walk_scene(K=200, L=10000, seed=3, iterations=30)  # M = 203,310
    return _WALK["sc"]


def test_mixed_walk_final_cost(zs_lib):
    sc = _walk()
    with _ba(0) as h:
        h.set_problem(sc)
        r64 = h.solve(sc.iterations)
    with _ba(1) as h:
        h.set_problem(sc)
        r32 = h.solve(sc.iterations)
        c = h.chi2()
    print("walk K=200 L=10000: fp64", r64.chi2_final, r64.attempts, "mixed", r32.chi2_final, r32.attempts,
          "cg", r32.refine_sweeps, "retries", r32.preconditioner_retries)
    assert r32.refine_sweeps >= r32.attempts - r32.cholesky_failures  # a CG iteration per solved attempt at least
    assert abs(r32.chi2_final - c) <= 1e-12 * c  # the reported cost is the state's
    assert abs(r32.chi2_final - r64.chi2_final) <= MIXED_COST_TOL * r64.chi2_final
    # this scene's late iterations reach a lambda where the FP32 factorisation of
    # the FP32-formed S fails (2 attempts measured): the retry path is exercised
    assert r32.preconditioner_retries >= 1


@pytest.mark.parametrize("lam_scale", [1e-3, 1e-7, 1e-9])
def test_mixed_steps_follow_fp64(zs_lib, lam_scale):
    """Single damped steps from one FP64 state at decreasing lambda (relative
    to the initial lambda, tau max diag H); the smallest are where the FP32
    factorisation of the FP32-formed S needs the shifted retry."""
    sc = _walk()
    with _ba(0) as h:
        h.set_problem(sc)
        h.solve(10)
        P, L = h.get_state()
        lam = lam_scale * h.initial_lambda()
        ref = h.linear_step(lam, want_S=False)
    with _ba(1) as h:
        h.set_problem(sc)
        h.set_state(P, L)
        mix = h.linear_step(lam, want_S=False)
    assert ref["ok"]
    assert mix["ok"]
    n = 6 * sc.K
    print("lam", lam, "step", rel_err(mix["delta"], ref["delta"]), "bs", rel_err(mix["bs"], ref["bs"]))
    assert rel_err(mix["delta"][:n], ref["delta"][:n]) < STEP_TOL
    assert rel_err(mix["delta"][n:], ref["delta"][n:]) < STEP_TOL
    assert rel_err(mix["bs"], ref["bs"]) < STEP_TOL


def test_mixed_deterministic(zs_lib):
    sc = scenes.walk_scene(K=200, L=6000, seed=8)
    outs = []
    for _ in range(2):
        with _ba(1) as h:
            h.set_problem(sc)
            rep = h.solve(8)
            outs.append((rep.chi2_final, rep.refine_sweeps, *h.get_state()))
    assert outs[0][:2] == outs[1][:2]
    assert np.array_equal(outs[0][2], outs[1][2]) and np.array_equal(outs[0][3], outs[1][3])


def test_mixed_degenerate_landmarks(zs_lib, oracle):
    """Fixed landmarks, a landmark seen once (singular H_ll block: zero
    inverse, as the reference) and landmarks without observations inside the
    operator's landmark chunks."""
    sc = scenes.arc_scene(12, 900, seed=31)
    sc.landmark_fixed[::7] = 1
    keep = np.ones(sc.M, dtype=bool)
    for l in (3, 50, 400):  # drop every observation of these landmarks
        keep &= sc.obs_landmark != l
    first = np.flatnonzero(sc.obs_landmark == 77)
    keep[first[1:]] = False  # landmark 77: a single observation
    sc.obs_pose, sc.obs_landmark, sc.obs_uv = sc.obs_pose[keep], sc.obs_landmark[keep], sc.obs_uv[keep]
    _, _, ro = oracle.solve(sc, 8)
    with _ba(1) as h:
        h.set_problem(sc)
        r = h.solve(8)
        P, L = h.get_state()
    assert abs(r.chi2_final - ro.chi2_final) <= MIXED_COST_TOL * ro.chi2_final
    for l in (3, 50, 400):
        assert np.array_equal(L[l], sc.landmarks[l])  # unobserved landmarks stay where they are


def test_mixed_robust_with_information(zs_lib, oracle):
    """The general operator (a robust weight W per observation): Huber loss and
    a 2 x 2 information matrix per observation, against the oracle: a single
    damped step, and the cost after 8 iterations (multi-step robust solves
    are compared at 1e-5, as for the plain form)."""
    sc = scenes.arc_scene(25, 2500, seed=3, huber=True)
    rng = np.random.default_rng(4)
    s = rng.uniform(0.5, 2.0, size=(sc.M, 1))
    sc.obs_info = np.concatenate([1.0 * s, 0.2 * s, 0.2 * s, 0.6 * s], axis=1)
    lam = oracle.initial_lambda(sc)
    o = oracle.linear_step(sc, lam, want_S=False)
    with _ba(1) as h:
        h.set_problem(sc)
        g = h.linear_step(lam, want_S=False)
    assert o["ok"] and g["ok"]
    assert rel_err(g["delta"], o["delta"]) < STEP_TOL
    _, _, ro = oracle.solve(sc, 8)
    with _ba(1) as h:
        h.set_problem(sc)
        r = h.solve(8)
    assert abs(r.chi2_final - ro.chi2_final) <= 1e-5 * ro.chi2_final


def test_mixed_blocked_preconditioner_ragged(zs_lib):
    """A mixed solve whose reduced system (n = 3600: 600 poses) takes the
    blocked tensor-core preconditioner with a 16-column last panel: the same
    accepted steps and the cost within the mixed form's 1e-6 of the FP64
    solve."""
    sc = scenes.walk_scene(K=600, L=20000, seed=71)  # M = 438,946
    res = []
    for precision in (0, 1):
        with _ba(precision) as h:
            h.set_problem(sc)
            res.append(h.solve(4))
    r64, r32 = res
    assert r32.accepted == r64.accepted and r32.cholesky_failures == 0
    assert abs(r32.chi2_final - r64.chi2_final) <= MIXED_COST_TOL * r64.chi2_final
