"""The window and graph of map::optimise (source/map.hpp:77-233) as the
library builds them (zs_map_optimise_plan: host code, no device) against the
oracle's restatement: the problem's poses, landmarks and edges, the frames
written back and the counts and outcome the reference prints, for the whole
map, local windows, the tracking mode and maps with missing frames. CPU."""

import numpy as np
import pytest

from zeroslam_gb300 import scenes


def _case_maps():
    sc = scenes.arc_scene(16, 900, seed=21, min_obs=2)
    cm = scenes.slam_map(sc)
    gone = scenes.slam_map(sc)
    gone.obs_frame = gone.obs_frame.copy()
    gone.obs_frame[::7] = -1
    return {"map": cm, "missing_frames": gone}


@pytest.mark.parametrize("lw,fixl", [(0, False), (2, False), (4, False), (6, False), (1, True), (3, True),
                                     (0, True)])
@pytest.mark.parametrize("which", ["map", "missing_frames"])
def test_plan_matches_oracle(zs_lib, oracle, lw, fixl, which):
    from zeroslam_gb300 import ba

    cm = _case_maps()[which]
    plan = ba.map_optimise_plan(cm, lw, fixl)
    _, _, info = oracle.map_optimise(cm, lw, fixl, 0)
    rep = plan["report"]
    assert (rep.frames, rep.landmarks, rep.edges) == (info["frames"], info["landmarks"], info["edges"])
    assert list(plan["pose_frame"]) == list(info["problem_frames"])
    assert list(plan["landmark_index"]) == list(info["problem_landmarks"])
    assert list(plan["edge_obs"]) == list(info["edge_obs"])
    assert rep.outcome == info["status"]
    if rep.outcome == ba.MAP_OPTIMISED:
        assert list(plan["written"]) == info["written"]


def test_plan_outcomes(zs_lib, oracle):
    from zeroslam_gb300 import ba

    cm = _case_maps()["map"]
    old = _case_maps()["map"]
    old.frame_id_generator = 1000  # every frame below the window
    p = ba.map_optimise_plan(old, 2, True)
    assert p["report"].outcome == ba.MAP_ALL_FIXED == oracle.map_optimise(old, 2, True, 0)[2]["status"]
    assert not p["written"].any()
    empty = scenes.CullMap(cm.frame_pose[:0], cm.frame_intrinsics[:0], cm.frame_id[:0], cm.landmark_id[:0],
                           cm.landmarks[:0], np.zeros(1, dtype=np.int64), cm.obs_frame[:0], cm.obs_frame_id[:0],
                           cm.obs_keypoint[:0], 0, 0)
    assert ba.map_optimise_plan(empty, 0, False)["report"].outcome == ba.MAP_NOTHING_TO_OPTIMISE
    bad = _case_maps()["map"]
    bad.obs_frame = bad.obs_frame.copy()
    bad.obs_frame[0] = bad.F
    with pytest.raises(ba.ZsError):
        ba.map_optimise_plan(bad, 0, False)


def _rotations(n, seed):
    """Random rotations over the whole group (uniform unit quaternions), so
    both branches of so3(rotation matrix) occur (trace <= 0 beyond 120 deg),
    plus the half-turns about each axis."""
    rng = np.random.default_rng(seed)
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q = np.concatenate([q, [[0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1], [1, 0, 0, 0]]])
    t = rng.normal(size=(q.shape[0], 3))
    return scenes.pack_poses(q, t)


def test_frame_pose_conversions_match_oracle(zs_lib, oracle):
    """zs_frame_to_pose / zs_pose_to_frame, bit for bit with the oracle's
    restatement (pinned to the reference in test_oracle_reference.py)."""
    from zeroslam_gb300 import ba

    poses = _rotations(500, 3)
    frames = oracle.pose_rt(poses)
    assert np.array_equal(ba.poses_to_frames(poses), frames)
    tr = frames[:, 0] + frames[:, 4] + frames[:, 8]
    assert (tr <= 0).sum() > 50 and (tr > 0).sum() > 50  # both branches
    assert np.array_equal(ba.frames_to_poses(frames), oracle.rt_pose(frames))
