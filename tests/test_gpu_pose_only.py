"""Pose-only bundle adjustment, zeroslam's tracking mode (every landmark fixed:
map optimise(1, true, 50), source/slam.hpp:316,387,469): the landmark blocks
vanish (zero H_ll inverses, no H_pl), S is block diagonal (one 6 x 6 block
per pose) and the solve reduces to independent pose updates. Single problems
in both forms and batched windows are compared with the oracle; the
one-launch paths (a single problem over the whole grid, a batch with one
CTA per window) with the oracle and with the general paths."""

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


# ---- batches of pose-only windows: one CTA per window ----


def _tracking_batch(seed):
    """Tracking windows of several shapes: one to four free poses among up
    to 32, a window with every pose fixed, a lone fixed pose and a window
    without observations (every landmark fixed throughout)."""
    rng = np.random.default_rng(seed)
    wins = []
    for i in range(10):
        k = int(rng.integers(2, 33))
        sc = _pose_only(scenes.arc_scene(k, int(rng.integers(200, 1500)), seed=seed + i))
        sc.pose_fixed[:] = 1
        free = rng.choice(k, size=min(k, 1 + i % 4), replace=False)
        sc.pose_fixed[free] = 0
        wins.append(sc)
    allfixed = _pose_only(scenes.arc_scene(6, 300, seed=seed + 20))
    allfixed.pose_fixed[:] = 1
    lone = _pose_only(scenes.arc_scene(1, 40, seed=seed + 21))
    empty = _pose_only(scenes.arc_scene(4, 50, seed=seed + 22))
    empty.obs_pose = empty.obs_pose[:0]
    empty.obs_landmark = empty.obs_landmark[:0]
    empty.obs_uv = empty.obs_uv[:0]
    return wins[:4] + [allfixed, lone] + wins[4:7] + [empty] + wins[7:]


def _run_batch(wins, iterations, precision=0, use_relative=False, **kw):
    with _ba(precision, **kw) as h:
        h.set_batch(wins)
        acc, reps, brep = h.solve_batch(iterations, use_relative)
        states = [h.get_window_state(w) for w in range(len(wins))]
    return acc, reps, brep, states


@pytest.mark.parametrize("use_relative", [False, True])
def test_windows_match_general_batch(zs_lib, use_relative):
    """The one-launch batch takes the general batched path's decisions in
    every window (same accepted steps, attempts, iterations and Cholesky
    failures) and reaches its cost and poses; empty and fully fixed windows
    report as the general path reports them."""
    wins = _tracking_batch(71)
    a1, r1, b1, s1 = _run_batch(wins, 30, use_relative=use_relative)
    a0, r0, b0, s0 = _run_batch(wins, 30, use_relative=use_relative, pose_only_path=0)
    assert b1.kernel_launches == 1 and b1.graph_launches == 0 and b0.graph_launches == 1
    assert a1 == a0
    for w in range(len(wins)):
        x, y = r1[w], r0[w]
        assert (x.accepted, x.attempts, x.iterations, x.cholesky_failures) == \
            (y.accepted, y.attempts, y.iterations, y.cholesky_failures), w
        assert abs(x.chi2_initial - y.chi2_initial) <= 1e-12 * abs(y.chi2_initial) + 1e-300, w
        assert abs(x.chi2_final - y.chi2_final) <= 1e-11 * abs(y.chi2_final) + 1e-300, w
        assert rel_err(s1[w][0], s0[w][0]) < 1e-9, w
        assert np.array_equal(s1[w][1], wins[w].landmarks)  # fixed landmarks do not move
        fixed = wins[w].pose_fixed.astype(bool)
        assert np.array_equal(s1[w][0][fixed], wins[w].poses[fixed]), w


def test_windows_against_oracle(zs_lib, oracle):
    """Every attempt's decision over the first three iterations (steps far
    above rounding: converged tracking problems reach trial steps that change
    the cost by ~1e-16 relative, where accept or reject follows the last bit
    of either implementation), and the cost and poses after twenty."""
    wins = _tracking_batch(73)[:6]
    _, reps, _, _ = _run_batch(wins, 3)
    _, reps20, _, states = _run_batch(wins, 20)
    for w, sc in enumerate(wins):
        _, _, ro = oracle.solve(sc, 3)
        r = reps[w]
        assert (r.accepted, r.attempts, r.iterations, r.cholesky_failures) == \
            (ro.accepted, ro.attempts, ro.iterations, ro.chol_failures), w
        poses, _, ro = oracle.solve(sc, 20)
        assert abs(reps20[w].chi2_final - ro.chi2_final) <= COST_TOL * ro.chi2_final + 1e-300, w
        assert rel_err(states[w][0], poses) < 1e-7, w


def test_windows_robust_information_and_forms(zs_lib):
    """Huber loss with information matrices, against the general batched
    path; the mixed-form handle takes the same FP64 path (identical bits)."""
    wins = []
    for i in range(6):
        sc = _pose_only(scenes.arc_scene(5 + i, 600, seed=80 + i, huber=True))
        sc.pose_fixed[:] = 1
        sc.pose_fixed[[0, 2 + i % 3]] = 0
        rng = np.random.default_rng(90 + i)
        s = rng.uniform(0.5, 2.0, size=(sc.M, 1))
        sc.obs_info = np.concatenate([1.0 * s, 0.2 * s, 0.2 * s, 0.6 * s], axis=1)
        wins.append(sc)
    _, r1, _, s1 = _run_batch(wins, 15)
    _, r0, _, _ = _run_batch(wins, 15, pose_only_path=0)
    _, rm, bm, sm = _run_batch(wins, 15, precision=1)
    assert bm.kernel_launches == 1
    for w in range(len(wins)):
        assert (r1[w].accepted, r1[w].attempts) == (r0[w].accepted, r0[w].attempts), w
        assert abs(r1[w].chi2_final - r0[w].chi2_final) <= 1e-11 * r0[w].chi2_final, w
        assert rm[w].chi2_final == r1[w].chi2_final and np.array_equal(sm[w][0], s1[w][0]), w
