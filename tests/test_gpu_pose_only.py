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
