"""Windowed bundle adjustment of a map (zeroslam_gb300/csrc/ba_map.cu,
zs_map_optimise) against map::optimise (source/map.hpp:65-267): the
reference's own outputs in tests/golden/map_optimise.npz and the oracle's
restatement (window selection, graph, frame conversion, solve, write-back)."""

import numpy as np
import pytest

from conftest import MAP_OPTIMISE_CASES, cull_from_npz, load_npz, map_state_cost, rel_err
from zeroslam_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ba(precision=0):
    from zeroslam_gb300 import ba

    return ba.BundleAdjuster(precision=precision)


@pytest.mark.parametrize("case", sorted(MAP_OPTIMISE_CASES))
def test_map_optimise_fixture(zs_lib, oracle, case):
    g = load_npz("map_optimise.npz")
    cm = cull_from_npz(g)
    lw, fixl, rounds = MAP_OPTIMISE_CASES[case]
    fo, Xo, info = oracle.map_optimise(cm, lw, fixl, rounds)
    with _ba() as h:
        fp, X, rep = h.map_optimise(cm, lw, fixl, rounds)
    assert rep.outcome == 0
    assert (rep.frames, rep.landmarks, rep.edges) == (info["frames"], info["landmarks"], info["edges"])
    assert rep.problem_poses == len(info["problem_frames"]) and rep.problem_landmarks == len(info["problem_landmarks"])
    tol = 1e-9 if rounds == 1 else 1e-6
    for want in ((fo, Xo), (g[f"{case}_frame_pose"], g[f"{case}_landmarks"])):
        assert rel_err(fp, want[0]) < tol
        assert rel_err(X, want[1]) < tol
    assert np.array_equal(cm.frame_pose, g["frame_pose"])  # the input map is untouched


@pytest.mark.parametrize("precision,lw", [(0, 0), (0, 4), (1, 0), (1, 4)])
def test_map_optimise_rounds(zs_lib, oracle, precision, lw):
    """Ten Huber rounds, global and windowed, FP64 and mixed: the cost of
    the written-back map on the window's problem agrees with the oracle's."""
    sc = scenes.arc_scene(15, 2000, seed=12, min_obs=2, **scenes.ADJOINT_INIT_NOISE)
    cm = scenes.slam_map(sc)
    fo, Xo, info = oracle.map_optimise(cm, lw, False, 10)
    with _ba(precision) as h:
        fp, X, rep = h.map_optimise(cm, lw, False, 10)
    assert rep.outcome == 0 and rep.solve.iterations >= 1
    c_o = map_state_cost(oracle, cm, info, fo, Xo)
    c = map_state_cost(oracle, cm, info, fp, X)
    assert abs(c - c_o) <= 1e-5 * c_o
    assert abs(rep.solve.chi2_final - c) <= 1e-9 * c  # the solve's cost is the written-back map's
    untouched = np.setdiff1d(np.arange(cm.L), info["problem_landmarks"])
    assert np.array_equal(X[untouched], cm.landmarks[untouched])


def test_map_optimise_outcomes(zs_lib):
    from zeroslam_gb300 import ba

    sc = scenes.arc_scene(6, 300, seed=14)
    cm = scenes.slam_map(sc)
    with _ba() as h:
        empty = scenes.CullMap(cm.frame_pose[:0], cm.frame_intrinsics[:0], cm.frame_id[:0], cm.landmark_id[:0],
                               cm.landmarks[:0], np.zeros(1, dtype=np.int64), cm.obs_frame[:0], cm.obs_frame_id[:0],
                               cm.obs_keypoint[:0], 0, 0)
        assert h.map_optimise(empty, 0, False, 5)[2].outcome == ba.MAP_NOTHING_TO_OPTIMISE
        old = scenes.slam_map(sc)
        old.frame_id_generator = 100  # every frame below the window: all fixed
        fp, X, rep = h.map_optimise(old, 1, True, 5)
        assert rep.outcome == ba.MAP_ALL_FIXED
        assert np.array_equal(fp, old.frame_pose) and np.array_equal(X, old.landmarks)
        bad = scenes.slam_map(sc)
        bad.obs_frame = bad.obs_frame.copy()
        bad.obs_frame[3] = bad.F
        with pytest.raises(ba.ZsError) as ex:
            h.map_optimise(bad, 0, False, 5)
        assert ex.value.status == ba.ZS_ERR_INVALID
        fp, X, rep = h.map_optimise(cm, 0, False, 3)  # the handle stays usable
        assert rep.outcome == ba.MAP_OPTIMISED


def test_map_optimise_then_resident_cull(zs_lib, oracle):
    """Global optimise, then zs_ba_cull on the solved window without a copy
    back: the same decisions as map::cull on the written-back map."""
    sc = scenes.arc_scene(10, 1500, seed=15, min_obs=2, **scenes.ADJOINT_INIT_NOISE)
    cm = scenes.slam_map(sc)
    with _ba() as h:
        fp, X, rep = h.map_optimise(cm, 0, False, 5)
        assert rep.problem_poses == cm.F and rep.problem_landmarks == cm.L
        e, m, crep = h.cull(cm.landmark_id, cm.frame_id, cm.landmark_id_generator, cm.frame_id_generator)
    after = scenes.slam_map(sc)
    after.frame_pose, after.landmarks = fp, X
    e_o, m_o, n_o = oracle.map_cull(after)
    assert np.array_equal(e, e_o) and np.array_equal(m.view(np.uint32), m_o.view(np.uint32))


def test_map_optimise_missing_frames(zs_lib, oracle):
    """Observations whose frame is not in the map are skipped (zeroslam's
    optimise requires every observing frame to be in the map): one round,
    global and windowed, against the oracle's restatement."""
    sc = scenes.arc_scene(12, 1200, seed=16, min_obs=2, **scenes.ADJOINT_INIT_NOISE)
    cm = scenes.slam_map(sc)
    cm.obs_frame = cm.obs_frame.copy()
    cm.obs_frame[::9] = -1
    for lw in (0, 4):
        fo, Xo, info = oracle.map_optimise(cm, lw, False, 1)
        with _ba() as h:
            fp, X, rep = h.map_optimise(cm, lw, False, 1)
        assert rep.edges == info["edges"] < int((cm.obs_frame >= 0).sum()) + 1
        assert rel_err(fp, fo) < 1e-9 and rel_err(X, Xo) < 1e-9
