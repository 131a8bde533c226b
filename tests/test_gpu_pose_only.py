"""Pose-only bundle adjustment, zeroslam's tracking mode (every landmark fixed:
map optimise(1, true, 50), source/slam.hpp:316,387,469): the landmark blocks
vanish (zero H_ll inverses, no H_pl), S is block diagonal (one 6 x 6 block
per pose) and the solve reduces to independent pose updates. Single problems
in both forms and batched windows are compared with the oracle."""

import numpy as np
import pytest

from conftest import rel_err
from zeroslam_gb300 import scenes

pytestmark = pytest.mark.gpu

COST_TOL = 1e-9
MIXED_COST_TOL = 1e-6


def _pose_only(sc):
    sc.landmark_fixed[:] = 1
    return sc


def _ba(precision, **kw):
    from zeroslam_gb300 import ba

    return ba.BundleAdjuster(precision=precision, **kw)


@pytest.mark.parametrize("precision", [0, 1])
def test_pose_only_single(zs_lib, oracle, precision):
    sc = _pose_only(scenes.arc_scene(12, 800, seed=41))
    poses_o, lms_o, ro = oracle.solve(sc, 10)
    with _ba(precision) as h:
        h.set_problem(sc)
        r = h.solve(10)
        P, L = h.get_state()
    tol = COST_TOL if precision == 0 else MIXED_COST_TOL
    assert abs(r.chi2_final - ro.chi2_final) <= tol * ro.chi2_final
    assert np.array_equal(L, sc.landmarks)  # fixed landmarks do not move
    if precision == 0:
        assert (r.accepted, r.attempts) == (ro.accepted, ro.attempts)
        assert rel_err(P, poses_o) < 1e-7


def test_pose_only_batch(zs_lib, oracle):
    wins = [_pose_only(w) for w in scenes.window_batch(5, seed=43, k_range=(3, 12), l_range=(100, 400))]
    for precision in (0, 1):
        with _ba(precision) as h:
            h.set_batch(wins)
            _, reps, _ = h.solve_batch(8)
        for w, sc in enumerate(wins):
            _, _, ro = oracle.solve(sc, 8)
            tol = COST_TOL if precision == 0 else MIXED_COST_TOL
            assert abs(reps[w].chi2_final - ro.chi2_final) <= tol * ro.chi2_final + 1e-12, (precision, w)


# ---- the one-launch path (every landmark fixed, at most 64 poses, at most 4 free) ----


def _tracking(seed, n_fixed=4, L=1500):
    """Tracking-shaped: one free pose among a few fixed ones, every landmark
    fixed (zeroslam's optimise(1, true, 50) after the window selection)."""
    sc = _pose_only(scenes.arc_scene(n_fixed + 1, L, seed=seed))
    sc.pose_fixed[:] = 1
    sc.pose_fixed[n_fixed // 2] = 0
    return sc


@pytest.mark.parametrize("precision", [0, 1])
def test_one_launch_against_oracle(zs_lib, oracle, precision):
    sc = _tracking(51)
    poses_o, _, ro = oracle.solve(sc, 50)
    with _ba(precision) as h:
        h.set_problem(sc)
        r = h.solve(50)
        P, L = h.get_state()
    assert r.kernel_launches == 1
    assert (r.accepted, r.attempts, r.iterations) == (ro.accepted, ro.attempts, ro.iterations)
    assert abs(r.chi2_final - ro.chi2_final) <= COST_TOL * ro.chi2_final
    assert rel_err(P, poses_o) < 1e-7
    assert np.array_equal(L, sc.landmarks)
    fixed = sc.pose_fixed.astype(bool)
    assert np.array_equal(P[fixed], sc.poses[fixed])  # fixed poses do not move


def test_one_launch_matches_general_path(zs_lib):
    """Same decisions as the general path (Schur, dense factor) on a pose-only
    problem with four free poses among twelve: every attempt's outcome, and
    the cost."""
    sc = _pose_only(scenes.arc_scene(12, 800, seed=53))
    sc.pose_fixed[:] = 1
    sc.pose_fixed[[2, 5, 7, 10]] = 0
    out = []
    for path in (1, 0):
        with _ba(0, pose_only_path=path) as h:
            h.set_problem(sc)
            r = h.solve(20)
            out.append((r, h.history(), h.get_state()[0]))
    (r1, h1, p1), (r0, h0, p0) = out
    assert r1.kernel_launches == 1 and r0.kernel_launches > 20
    assert (r1.accepted, r1.attempts) == (r0.accepted, r0.attempts)
    assert [(a["solved"], a["accepted"]) for a in h1] == [(a["solved"], a["accepted"]) for a in h0]
    assert abs(r1.chi2_final - r0.chi2_final) <= 1e-12 * r0.chi2_final
    assert rel_err(p1, p0) < 1e-10


def test_one_launch_robust_information(zs_lib, oracle):
    """Huber loss and per-observation information matrices, against the oracle."""
    sc = _pose_only(scenes.arc_scene(8, 1200, seed=57, huber=True))
    sc.pose_fixed[:] = 1
    sc.pose_fixed[[1, 4, 6]] = 0
    rng = np.random.default_rng(58)
    s = rng.uniform(0.5, 2.0, size=(sc.M, 1))
    sc.obs_info = np.concatenate([1.0 * s, 0.2 * s, 0.2 * s, 0.6 * s], axis=1)
    _, _, ro = oracle.solve(sc, 10)
    with _ba(0) as h:
        h.set_problem(sc)
        r = h.solve(10)
    assert r.kernel_launches == 1
    assert (r.accepted, r.attempts) == (ro.accepted, ro.attempts)
    assert abs(r.chi2_final - ro.chi2_final) <= COST_TOL * ro.chi2_final


def test_one_launch_repeats_and_limits(zs_lib):
    """Bit-for-bit repetition; more than 64 poses, or more than 4 free ones,
    take the general path."""
    sc = _tracking(59)
    res = []
    for _ in range(2):
        with _ba(0) as h:
            h.set_problem(sc)
            r = h.solve(50)
            res.append((r.chi2_final, h.get_state()[0].copy()))
    assert res[0][0] == res[1][0] and np.array_equal(res[0][1], res[1][1])
    big = _pose_only(scenes.arc_scene(70, 600, seed=61))
    with _ba(0) as h:
        h.set_problem(big)
        r = h.solve(3)
    assert r.kernel_launches > 1 and r.accepted >= 1
    five = _pose_only(scenes.arc_scene(8, 600, seed=63))
    five.pose_fixed[:] = 1
    five.pose_fixed[1:6] = 0
    with _ba(0) as h:
        h.set_problem(five)
        r = h.solve(3)
    assert r.kernel_launches > 1 and r.accepted >= 1
