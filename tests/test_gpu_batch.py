"""Batched local windows (zs_ba_set_batch / zs_ba_solve_batch): every window
of a batch must follow the same LM path as its own factor_graph::solve.

FP64 batches are compared window by window with the oracle (accepted steps,
attempts, iterations and the final cost to 1e-9 relative, the state to 1e-7)
and with single-problem solves; the mixed form is compared with the FP64
batch on the final cost (1e-6 relative). The graph launch (conditional WHILE
node) and the host loop over rounds must give identical bits."""

import numpy as np
import pytest

from conftest import rel_err
from zeroslam_gb300 import scenes

pytestmark = pytest.mark.gpu

COST_TOL = 1e-9
STATE_TOL = 1e-7
MIXED_COST_TOL = 1e-6


def _ba(precision=0, **kw):
    from zeroslam_gb300 import ba

    return ba.BundleAdjuster(precision=precision, **kw)


def _small_batch(n=7, seed=5):
    return scenes.window_batch(n, seed=seed, k_range=(3, 14), l_range=(60, 400))


def _run(wins, iterations=10, precision=0, use_relative=False, **kw):
    with _ba(precision, **kw) as h:
        h.set_batch(wins)
        acc, reps, brep = h.solve_batch(iterations, use_relative)
        states = [h.get_window_state(w) for w in range(len(wins))]
    return acc, reps, brep, states


@pytest.mark.parametrize("use_relative", [False, True])
def test_batch_fp64_matches_oracle(zs_lib, oracle, use_relative):
    wins = _small_batch()
    acc, reps, brep, states = _run(wins, 10, use_relative=use_relative)
    assert brep.graph_launches == 1 and brep.windows == len(wins)
    total = 0
    for w, sc in enumerate(wins):
        poses, lms, ro = oracle.solve(sc, 10, use_relative)
        r = reps[w]
        assert (r.accepted, r.attempts, r.iterations) == (ro.accepted, ro.attempts, ro.iterations), w
        assert r.cholesky_failures == ro.chol_failures
        assert abs(r.chi2_initial - ro.chi2_initial) <= 1e-12 * ro.chi2_initial
        assert abs(r.chi2_final - ro.chi2_final) <= COST_TOL * ro.chi2_final, (w, r.chi2_final, ro.chi2_final)
        assert rel_err(states[w][0], poses) < STATE_TOL
        assert rel_err(states[w][1], lms) < STATE_TOL
        total += ro.accepted
    assert acc == total


def test_batch_matches_single_solves(zs_lib):
    wins = _small_batch(5, seed=11)
    _, reps, _, states = _run(wins, 8)
    for w, sc in enumerate(wins):
        with _ba() as h:
            h.set_problem(sc)
            r1 = h.solve(8)
            p1, l1 = h.get_state()
        r = reps[w]
        assert (r.accepted, r.attempts) == (r1.accepted, r1.attempts)
        assert abs(r.chi2_final - r1.chi2_final) <= COST_TOL * r1.chi2_final
        assert rel_err(states[w][0], p1) < STATE_TOL and rel_err(states[w][1], l1) < STATE_TOL


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_graph_equals_host_loop(zs_lib, precision):
    wins = _small_batch(6, seed=7)
    a = _run(wins, 10, precision, batch_graph=1)
    b = _run(wins, 10, precision, batch_graph=0)
    assert a[2].graph_launches == 1 and b[2].graph_launches == 0
    assert a[2].rounds == b[2].rounds
    for w in range(len(wins)):
        assert a[1][w].chi2_final == b[1][w].chi2_final
        assert np.array_equal(a[3][w][0], b[3][w][0]) and np.array_equal(a[3][w][1], b[3][w][1])


def test_batch_deterministic_and_reusable(zs_lib):
    wins = _small_batch(6, seed=9)
    with _ba(1) as h:
        h.set_batch(wins)
        _, r1, _ = h.solve_batch(10)
        s1 = [h.get_window_state(w) for w in range(len(wins))]
        h.reset_state()
        _, r2, _ = h.solve_batch(10)  # same graph, relaunched
        s2 = [h.get_window_state(w) for w in range(len(wins))]
    for w in range(len(wins)):
        assert r1[w].chi2_final == r2[w].chi2_final
        assert np.array_equal(s1[w][0], s2[w][0]) and np.array_equal(s1[w][1], s2[w][1])


def test_batch_mixed_final_cost(zs_lib):
    wins = scenes.window_batch(12, seed=3)  # the full size range: K in [5, 30], L in [200, 3000]
    _, r64, _, _ = _run(wins, 10, 0)
    _, r32, brep, _ = _run(wins, 10, 1)
    for w in range(len(wins)):
        assert abs(r32[w].chi2_final - r64[w].chi2_final) <= MIXED_COST_TOL * r64[w].chi2_final, w
    assert sum(brep.bucket_windows) == len(wins)
    assert all(t in (64, 128, 256, 512, 1024) for t, c in zip(brep.bucket_threads, brep.bucket_windows) if c)


def test_batch_uneven_and_degenerate_windows(zs_lib, oracle):
    wins = _small_batch(4, seed=13)
    lone = scenes.arc_scene(1, 30, seed=2)  # a single (fixed) pose
    empty = scenes.arc_scene(4, 50, seed=3)
    empty.obs_pose = empty.obs_pose[:0]
    empty.obs_landmark = empty.obs_landmark[:0]
    empty.obs_uv = empty.obs_uv[:0]
    big = scenes.arc_scene(32, 600, seed=4)  # the largest window size (n = 192)
    wins = [wins[0], lone, wins[1], empty, big, wins[2]]
    acc, reps, brep, states = _run(wins, 6)
    assert reps[3].iterations == 0 and reps[3].accepted == 0
    assert np.array_equal(states[3][0], empty.poses) and np.array_equal(states[3][1], empty.landmarks)
    for w in (0, 1, 2, 4, 5):
        _, _, ro = oracle.solve(wins[w], 6)
        assert reps[w].accepted == ro.accepted
        # the single-pose window converges to a cost at rounding level (~1e-20)
        assert abs(reps[w].chi2_final - ro.chi2_final) <= COST_TOL * ro.chi2_final + 1e-12


def test_batch_rejects_oversized_and_mixed_cameras(zs_lib):
    from zeroslam_gb300 import ba

    with _ba() as h:
        with pytest.raises(ba.ZsError):
            h.set_batch([scenes.arc_scene(33, 100, seed=1)])
        a = scenes.arc_scene(5, 100, seed=1)
        b = scenes.arc_scene(5, 100, seed=2)
        b.intrinsics = (500.0, 500.0, 320.0, 240.0)
        with pytest.raises(ba.ZsError):
            h.set_batch([a, b])
        h.set_batch([a])
        with pytest.raises(ba.ZsError):
            h.solve(3)  # single-problem entry points refuse a batch


def test_batch_autotune_cache_file(zs_lib, tmp_path):
    import json

    path = tmp_path / "tune.json"
    wins = _small_batch(4, seed=21)
    with _ba(1, autotune_cache=str(path).encode()) as h:
        h.set_batch(wins)
        _, _, brep = h.solve_batch(3)
    d = json.loads(path.read_text())
    used = [b for b, c in enumerate(brep.bucket_windows) if c]
    got = {(e["precision"], e["bucket"]): e["threads"] for e in d["entries"]}
    for b in used:
        assert got[("mixed", b)] == brep.bucket_threads[b]


def test_batch_huber_windows(zs_lib, oracle):
    """Local windows as map::optimise builds them, with loss_huber(sqrt(5.991))
    (source/map.hpp:74): the FP64 batch against the oracle window by window
    after one iteration (1e-9). After five, the FP64 batch, the mixed batch
    and the single-problem FP64 solve all lower the cost and stay within 5% of
    the oracle's: under Huber the outliers' second-order term is switched by
    the sign of rho' + 2 rho'' e^2, zero in exact arithmetic, so states that
    differ in the last bits (the dense solves sum in different orders; the
    host's libm and the device's sin and cos round differently) take
    different branches and the paths separate into nearby minima (measured:
    up to 1.9e-4 on most windows, 2.8e-2 on one, where the oracle built on
    aarch64 and on x86-64 themselves end 2.9e-2 apart)."""
    wins = _small_batch(6, seed=9)
    for w in wins:
        w.loss_kind, w.loss_delta = 1, float(np.sqrt(5.991))
    _, reps1, _, _ = _run(wins, 1)
    _, reps, _, _ = _run(wins, 5)
    _, reps_m, _, _ = _run(wins, 5, precision=1)
    for w, sc in enumerate(wins):
        _, _, ro1 = oracle.solve(sc, 1)
        assert abs(reps1[w].chi2_final - ro1.chi2_final) <= COST_TOL * ro1.chi2_final, (w, reps1[w].chi2_final)
        _, _, ro = oracle.solve(sc, 5)
        with _ba() as h:
            h.set_problem(sc)
            rs = h.solve(5)
        for c in (reps[w].chi2_final, reps_m[w].chi2_final, rs.chi2_final):
            assert abs(c - ro.chi2_final) <= 5e-2 * ro.chi2_final, (w, c, ro.chi2_final)
            assert c < ro.chi2_initial
