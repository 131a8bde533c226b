"""Map culling on the device (zeroslam_gb300/csrc/ba_cull.cu, zs_map_cull and
zs_ba_cull) against the oracle's restatement of map::cull
(source/map.hpp:269-323): the erase decisions and the float mean errors
must be equal bit for bit, on maps where every branch of the cull occurs, on
the reference's own fixtures and known answers, and on the resident state
of a solve."""

import numpy as np
import pytest

from conftest import CULL_FIXTURES, cull_boundary_maps, cull_from_npz, known_answer_cull_maps, load_npz
from zeroslam_gb300 import scenes

pytestmark = pytest.mark.gpu


def _ba(precision=0):
    from zeroslam_gb300 import ba

    return ba.BundleAdjuster(precision=precision)


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


@pytest.mark.parametrize("name", CULL_FIXTURES)
def test_map_cull_fixtures(zs_lib, oracle, name):
    g = load_npz(name)
    cm = cull_from_npz(g)
    e_o, m_o, n_o = oracle.map_cull(cm)
    with _ba() as h:
        e, m, rep = h.map_cull(cm)
    assert np.array_equal(e, g["ref_erase"])
    assert _same(m, m_o)
    assert rep.erased == n_o and rep.error_passes == int((m_o >= 0).sum())


@pytest.mark.parametrize("case", known_answer_cull_maps(), ids=lambda c: c[0])
def test_map_cull_known_answers(zs_lib, case):
    _, cm, want = case
    with _ba() as h:
        e, _, rep = h.map_cull(cm)
    assert int(e[0]) == want and rep.erased == want


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_map_cull_random_maps(zs_lib, oracle, seed):
    sc = scenes.arc_scene(20, 4000, seed=80 + seed)
    with _ba() as h:
        for cm in (scenes.cull_map(sc, seed=seed, truth=True), scenes.cull_map(sc, seed=seed)):
            e_o, m_o, n_o = oracle.map_cull(cm)
            e, m, rep = h.map_cull(cm)
            assert np.array_equal(e, e_o) and _same(m, m_o) and rep.erased == n_o


def test_map_cull_walk_scale(zs_lib, oracle):
    """The 1M-observation walk as a map (ground truth, all branches)."""
    sc = scenes.walk_scene(seed=1)
    cm = scenes.cull_map(sc, seed=5, truth=True)
    e_o, m_o, n_o = oracle.map_cull(cm)
    with _ba() as h:
        e, m, rep = h.map_cull(cm)
        e2, m2, _ = h.map_cull(cm)  # the buffers are reused
    assert cm.M > 500000
    assert np.array_equal(e, e_o) and _same(m, m_o) and rep.erased == n_o
    assert np.array_equal(e, e2) and _same(m, m2)


def test_map_cull_empty_and_invalid(zs_lib):
    from zeroslam_gb300 import ba

    sc = scenes.arc_scene(6, 200, seed=90)
    cm = scenes.cull_map(sc, seed=0, truth=True)
    empty = scenes.CullMap(cm.frame_pose[:0], cm.frame_intrinsics[:0], cm.frame_id[:0], cm.landmark_id[:0],
                           cm.landmarks[:0], np.zeros(1, dtype=np.int64), cm.obs_frame[:0], cm.obs_frame_id[:0],
                           cm.obs_keypoint[:0], 0, 0)
    with _ba() as h:
        e, m, rep = h.map_cull(empty)
        assert e.shape == (0,) and rep.erased == 0
        bad = scenes.cull_map(sc, seed=0, truth=True)
        bad.obs_frame = bad.obs_frame.copy()
        bad.obs_frame[bad.obs_frame >= 0] = bad.F  # one past the last frame: rejected, not read
        bad.landmark_id_generator = 0  # every landmark reaches the error pass
        bad.frame_id_generator = 0
        with pytest.raises(ba.ZsError) as ex:
            h.map_cull(bad)
        assert ex.value.status == ba.ZS_ERR_INVALID
        e, m, rep = h.map_cull(cm)  # the handle stays usable
        assert rep.erased > 0


@pytest.mark.parametrize("precision", [0, 1])
def test_resident_cull_after_solve(zs_lib, oracle, precision):
    """zs_ba_cull on the solved state = map::optimise's write-back (the
    oracle's so3 matrix of each pose) followed by map::cull."""
    sc = scenes.arc_scene(15, 3000, seed=95)
    # every 10th landmark's observations pulled 15 px apart, alternately left
    # and right: no landmark position fits them, so they stay above 5.991
    far = np.flatnonzero(sc.obs_landmark % 10 == 0)
    sc.obs_uv[far, 0] += np.where(np.arange(far.size) % 2 == 0, 15.0, -15.0)
    sc.obs_uv = sc.obs_uv.astype(np.float32).astype(np.float64)  # keypoints are float
    lm_id = np.arange(sc.L, dtype=np.int32) + 1000
    fr_id = np.arange(sc.K, dtype=np.int32) + 10
    gens = [(1000, 10), (1000 + sc.L // 2 + 500, 10 + sc.K + 3)]
    with _ba(precision) as h:
        h.set_problem(sc)
        h.solve(5)
        P, Lm = h.get_state()
        out = [h.cull(lm_id, fr_id, lg, fg) for lg, fg in gens]
    solved = sc.copy()
    solved.poses, solved.landmarks = P, Lm
    cm = scenes.cull_map(solved, plain=True, frame_pose=oracle.pose_rt(P))
    for (lg, fg), (e, m, rep) in zip(gens, out):
        cm.landmark_id_generator, cm.frame_id_generator = lg, fg
        e_o, m_o, n_o = oracle.map_cull(cm)
        assert np.array_equal(e, e_o) and _same(m, m_o) and rep.erased == n_o
        assert 0 < n_o < sc.L


def test_map_cull_boundaries(zs_lib, oracle):
    """The cull's id, recency and depth boundaries: decisions and means as
    the oracle's (pinned to the reference on the same maps)."""
    with _ba() as h:
        for cm, want in cull_boundary_maps():
            e, m, _ = h.map_cull(cm)
            e_o, m_o, _ = oracle.map_cull(cm)
            assert int(e[0]) == int(e_o[0]) == want and _same(m, m_o)
