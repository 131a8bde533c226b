"""The oracle's host threads and its iteration-by-iteration solve change no
result: linear steps, Cholesky factors (with and without a failed pivot) and
whole solves are bit-for-bit those of one thread, and the stepwise solve is
the solve."""

import numpy as np

from zeroslam_gb300 import scenes


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def test_threads_bit_identical(oracle):
    sc = scenes.arc_scene(30, 3000, seed=3, huber=True)
    keep = oracle.threads
    try:
        oracle.set_threads(1)
        lam = oracle.initial_lambda(sc)
        a = oracle.linear_step(sc, lam)
        p1, l1, r1 = oracle.solve(sc, 4)
        oracle.set_threads(7)
        b = oracle.linear_step(sc, lam)
        p2, l2, r2 = oracle.solve(sc, 4)
        for k in ("S", "bs", "delta", "b", "hpp", "hll"):
            assert np.array_equal(_bits(a[k]), _bits(b[k])), k
        assert np.array_equal(_bits(p1), _bits(p2)) and np.array_equal(_bits(l1), _bits(l2))
        assert (r1.attempts, r1.accepted, r1.chi2_final) == (r2.attempts, r2.accepted, r2.chi2_final)
        rng = np.random.default_rng(0)
        for n, bad in ((1, None), (64, None), (65, None), (300, 250), (700, None)):
            G = rng.normal(size=(n, n))
            A = G @ G.T + np.eye(n)
            if bad is not None:
                A[bad, bad] = -1.0
            oracle.set_threads(1)
            ok1, L1 = oracle.cholesky(A)
            oracle.set_threads(5)
            ok2, L2 = oracle.cholesky(A)
            assert ok1 == ok2 == (bad is None) and np.array_equal(_bits(L1), _bits(L2)), n
    finally:
        oracle.set_threads(keep)


def test_stepwise_is_the_solve(oracle):
    for sc, iters in ((scenes.arc_scene(12, 800, seed=5, huber=True), 6), (scenes.small_scene(), 10)):
        p1, l1, r1 = oracle.solve(sc, iters)
        st = oracle.stepwise(sc)
        done = 0
        while done < iters and st.iteration():
            done += 1
        p2, l2, r2 = st.finish()
        assert np.array_equal(p1, p2) and np.array_equal(l1, l2)
        assert (r1.iterations, r1.accepted, r1.attempts, r1.chi2_final) == \
            (r2.iterations, r2.accepted, r2.attempts, r2.chi2_final)
