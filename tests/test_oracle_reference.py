"""The oracle against zeroslam's solver run live (only where the reference
tree has been compiled into oracle/_ref; skipped elsewhere)."""

import numpy as np
import pytest

from conftest import rel_err
from zeroslam_gb300 import scenes


def test_chi2_bitwise(oracle, reference):
    sc = scenes.arc_scene(10, 300, seed=21)
    assert oracle.chi2(sc) == reference.chi2(sc)


@pytest.mark.parametrize("seed,huber", [(31, False), (32, True)])
def test_single_step_parity(oracle, reference, seed, huber):
    sc = scenes.arc_scene(15, 800, seed=seed, huber=huber)
    po, lo, rep = oracle.solve(sc, 1)
    pr, lr, acc, c0, c1, _, _ = reference.solve(sc, 1)
    assert rep.accepted == acc
    assert rel_err(po - sc.poses, pr - sc.poses) < 1e-9
    assert rel_err(lo - sc.landmarks, lr - sc.landmarks) < 1e-9
    assert abs(rep.chi2_final - c1) <= 1e-9 * c1


def test_full_solve_parity_window(oracle, reference):
    sc = scenes.arc_scene(12, 1200, seed=41)
    po, lo, rep = oracle.solve(sc, 10)
    pr, lr, acc, c0, c1, _, _ = reference.solve(sc, 10)
    assert rep.accepted == acc
    assert abs(rep.chi2_final - c1) <= 1e-9 * c1
    assert rel_err(po, pr) < 1e-8


def test_cauchy_tukey_parity(oracle, reference):
    for kind in (2, 3):
        sc = scenes.arc_scene(8, 300, seed=50 + kind)
        sc.loss_kind, sc.loss_delta = kind, 2.0
        po, lo, rep = oracle.solve(sc, 3)
        pr, lr, acc, c0, c1, _, _ = reference.solve(sc, 3)
        assert rep.accepted == acc
        assert abs(rep.chi2_final - c1) <= 1e-9 * abs(c1)


def test_random_cholesky_and_invert(oracle, reference):
    rng = np.random.default_rng(7)
    for n in (3, 17, 64):
        G = rng.normal(size=(n, n))
        A = G @ G.T + np.eye(n)
        ok1, L1 = oracle.cholesky(A)
        ok2, L2 = reference.cholesky(A)
        assert ok1 and ok2 and np.array_equal(L1, L2)
    for _ in range(20):
        A = rng.normal(size=(3, 3))
        assert np.array_equal(oracle.invert3(A)[1], reference.invert3(A)[1])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_map_cull_parity(oracle, reference, seed):
    """map::cull run live on maps built by scenes.cull_map (every branch
    made to occur) and on a plain walk map, against the restatement."""
    from conftest import known_answer_cull_maps

    sc = scenes.arc_scene(12, 1500, seed=70 + seed)
    for cm in (scenes.cull_map(sc, seed=seed, truth=True), scenes.cull_map(sc, seed=seed)):
        e, _, n = oracle.map_cull(cm)
        er, nr = reference.map_cull(cm)
        assert np.array_equal(e, er) and n == nr
    for _, cm, want in known_answer_cull_maps():
        er, nr = reference.map_cull(cm)
        assert int(er[0]) == want
    assert np.array_equal(oracle.pose_rt(sc.poses), reference.pose_rt(sc.poses))


def test_map_optimise_parity(oracle, reference):
    """map::optimise live: one round of the global and windowed graphs to
    rounding; ten rounds under the Huber loss by cost (the reference's vertex
    order comes from hash sets, so weakly seen landmarks drift apart at the
    level of the robust solve's rounding, as for multi-step robust solves);
    the tracking mode to 1e-6."""
    from conftest import map_state_cost

    sc = scenes.arc_scene(12, 1200, seed=9, min_obs=2, **scenes.ADJOINT_INIT_NOISE)
    cm = scenes.slam_map(sc)
    assert np.array_equal(oracle.rt_pose(cm.frame_pose), reference.rt_pose(cm.frame_pose))
    for lw in (0, 4):
        fo, Xo, info = oracle.map_optimise(cm, lw, False, 1)
        fr, Xr = reference.map_optimise(cm, lw, False, 1)
        assert rel_err(fo, fr) < 1e-12 and rel_err(Xo, Xr) < 1e-12
        fo, Xo, info = oracle.map_optimise(cm, lw, False, 10)
        fr, Xr = reference.map_optimise(cm, lw, False, 10)
        co, cr = map_state_cost(oracle, cm, info, fo, Xo), map_state_cost(oracle, cm, info, fr, Xr)
        assert abs(co - cr) <= 1e-5 * cr
    fo, Xo, _ = oracle.map_optimise(cm, 1, True, 50)
    fr, Xr = reference.map_optimise(cm, 1, True, 50)
    assert rel_err(fo, fr) < 1e-6 and np.array_equal(Xo, Xr)


@pytest.mark.parametrize("seed", [0, 1])
def test_find_matches_parity(oracle, reference, seed):
    from conftest import known_answer_descriptors

    lhs, rhs = scenes.descriptor_pair(400, 500, seed=10 + seed)
    for thr, k, size in [(32.0, 2, 1000), (64.0, 4, 1601), (128.0, 8, 4000), (float("nan"), 2, 100), (-1.0, 1, 100)]:
        a = oracle.find_matches(lhs, rhs, thr, k, size)
        b = reference.find_matches(lhs, rhs, thr, k, size)
        assert np.array_equal(a, b)
    onehot, (l, r, thr, k, size, want) = known_answer_descriptors()
    assert len(reference.find_matches(l, r, thr, k, size)) == want
    m = reference.find_matches(onehot, np.zeros((1, 32), dtype=np.uint8), 2.0, 1, 256)
    assert len(m) == 256 and np.all(m["score"] == 1.0)


def test_solve_parity_k50_and_windows(oracle, reference):
    """The oracle against the reference on a 50-keyframe scene (the
    differentiable configuration's size) and on windows of the batched
    configuration, over whole solves."""
    sc = scenes.arc_scene(50, 1500, seed=51)
    po, lo, rep = oracle.solve(sc, 3)
    pr, lr, acc, c0, c1, _, _ = reference.solve(sc, 3)
    assert rep.accepted == acc and abs(rep.chi2_final - c1) <= 1e-9 * c1
    assert rel_err(po, pr) < 1e-8 and rel_err(lo, lr) < 1e-8
    for w in (scenes.window_batch(256)[i] for i in (0, 2)):
        po, lo, rep = oracle.solve(w, 10)
        pr, lr, acc, c0, c1, _, _ = reference.solve(w, 10)
        assert rep.accepted == acc and abs(rep.chi2_final - c1) <= 1e-9 * c1
        assert rel_err(po, pr) < 1e-8


def test_frame_pose_conversions_parity(oracle, reference):
    """so3 from a rotation matrix and back (source/lie.hpp:159-204) over the
    whole rotation group, both branches of the trace test, bit for bit."""
    import numpy as np

    rng = np.random.default_rng(5)
    q = rng.normal(size=(400, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    poses = scenes.pack_poses(q, rng.normal(size=(400, 3)))
    frames = reference.pose_rt(poses)
    assert np.array_equal(oracle.pose_rt(poses), frames)
    assert np.array_equal(oracle.rt_pose(frames), reference.rt_pose(frames))
    assert (frames[:, 0] + frames[:, 4] + frames[:, 8] <= 0).sum() > 50


def test_map_cull_parity_large(oracle, reference):
    """map::cull on an 844,142-observation map with every landmark in the
    error pass (both id generators 0), landmark for landmark."""
    sc = scenes.arc_scene(60, 20000, seed=99)
    cm = scenes.cull_map(sc, seed=4, truth=True)
    cm.landmark_id_generator = 0
    cm.frame_id_generator = 0
    e, _, n = oracle.map_cull(cm)
    er, nr = reference.map_cull(cm)
    assert cm.M > 800000 and n == nr > 0 and np.array_equal(e, er)


def test_map_cull_boundaries(oracle, reference):
    """map::cull's id, recency and depth boundaries and a NaN location,
    oracle against the reference."""
    from conftest import cull_boundary_maps

    maps = [cm for cm, _ in cull_boundary_maps()]
    nan = cull_boundary_maps()[2][0]
    nan.landmarks = np.array([[np.nan, 0.0, 1.0]])
    for cm in maps + [nan]:
        e, _, _ = oracle.map_cull(cm)
        er, _ = reference.map_cull(cm)
        assert np.array_equal(e, er)
    assert int(oracle.map_cull(nan)[0][0]) == 0  # a NaN mean is not >= 5.991


def test_find_matches_random_trials(oracle, reference):
    """Small random trials over sizes, thresholds (including non-integers),
    k and capacities, with descriptors drawn from few distinct values so that
    ties are frequent; oracle and reference match for match."""
    rng = np.random.default_rng(12)
    for _ in range(40):
        nl, nr = int(rng.integers(0, 40)), int(rng.integers(0, 40))
        pool = rng.integers(0, 256, size=(6, 32), dtype=np.uint8)
        lhs = pool[rng.integers(0, 6, nl)] ^ (rng.random((nl, 32)) < 0.02).astype(np.uint8)
        rhs = pool[rng.integers(0, 6, nr)] ^ (rng.random((nr, 32)) < 0.02).astype(np.uint8)
        thr = float(rng.choice([0.0, 1.0, 5.5, 32.0, 129.0, 300.0]))
        k = int(rng.integers(1, 9))
        size = int(rng.integers(0, 3 * max(nl, 1) * k))
        assert np.array_equal(oracle.find_matches(lhs, rhs, thr, k, size), reference.find_matches(lhs, rhs, thr, k, size))
