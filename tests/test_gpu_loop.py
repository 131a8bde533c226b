"""The 1000-keyframe loop (configuration 4: 200,000 landmarks, ~4M
observations, a dense 6000 x 6000 reduced camera system) against the
oracle: one FP64 linear step at the oracle's initial damping (b, b_s and the
step to 1e-9), three LM iterations in FP64 (accepted steps, attempts, cost to
1e-9) and in the mixed form (cost to 1e-6 of the oracle's), and the dense
solve at n = 6000 in both precisions against numpy. These reach the
n = 6000 code paths: the FP64 factorisation's 188 panels, the mixed form's
blocked preconditioner factor over 94 panels and the deepest levels of its
recursive L^-1."""

import numpy as np
import pytest

from conftest import rel_err
from zeroslam_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def loop():
    return scenes.loop_large_scene()


def test_loop_linear_step_fp64(zs_lib, oracle, loop):
    from zeroslam_gb300 import ba

    lam = oracle.initial_lambda(loop)
    o = oracle.linear_step(loop, lam, want_S=False)
    with ba.BundleAdjuster(precision=ba.FP64) as h:
        h.set_problem(loop)
        assert abs(h.initial_lambda() - lam) <= 1e-13 * lam
        assert abs(h.chi2() - oracle.chi2(loop)) <= 1e-12 * oracle.chi2(loop)
        g = h.linear_step(lam, want_S=False)
    assert o["ok"] and g["ok"]
    n = 6 * loop.K
    assert rel_err(g["b"], o["b"]) < 1e-9
    assert rel_err(g["bs"], o["bs"]) < 1e-9
    assert rel_err(g["delta"], o["delta"]) < 1e-9
    assert rel_err(g["delta"][:n], o["delta"][:n]) < 1e-9


def test_loop_three_iterations(zs_lib, oracle, loop):
    from zeroslam_gb300 import ba

    _, _, ro = oracle.solve(loop, 3)
    assert ro.iterations == 3
    with ba.BundleAdjuster(precision=ba.FP64) as h:
        h.set_problem(loop)
        r = h.solve(3)
    assert (r.accepted, r.attempts, r.cholesky_failures) == (ro.accepted, ro.attempts, ro.chol_failures)
    assert abs(r.chi2_initial - ro.chi2_initial) <= 1e-12 * ro.chi2_initial
    assert abs(r.chi2_final - ro.chi2_final) <= 1e-9 * ro.chi2_final
    with ba.BundleAdjuster(precision=ba.MIXED) as h:
        h.set_problem(loop)
        rm = h.solve(3)
        cm = h.chi2()
    assert rm.accepted == ro.accepted
    assert abs(rm.chi2_final - cm) <= 1e-12 * cm
    assert abs(cm - ro.chi2_final) <= 1e-6 * ro.chi2_final


def test_dense_cholesky_6000(zs_lib):
    """zs_dense_cholesky_solve at the loop's reduced-system size, both
    precisions, against numpy's factor and solve."""
    from zeroslam_gb300 import ba

    n = 6000
    rng = np.random.default_rng(6000)
    G = rng.normal(size=(n, n))
    A = G @ G.T / n + np.eye(n)
    b = rng.normal(size=n)
    ok, Lg, x = ba.dense_cholesky_solve(A, b)
    assert ok
    assert rel_err(Lg, np.linalg.cholesky(A)) < 1e-12
    xr = np.linalg.solve(A, b)
    assert rel_err(x, xr) < 1e-11
    ok, _, xm = ba.dense_cholesky_solve(A, b, precision=ba.MIXED)
    assert ok and rel_err(xm, xr) < 1e-10
