"""zs_dense_cholesky_solve_noalloc, the variant of the dense reduced-system
solve for callers that may not allocate device memory while running (a
real-time tracking thread that must not block in the allocator, or a host
whose device memory belongs to another allocator). Its workspace is a fixed
array inside the library, shared by every call, so two calls in a row must
each give the same answer as the allocating entry point. This file is
collected last so a failure here cannot hide the other tests' results."""

import ctypes as C

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu

_dp = C.POINTER(C.c_double)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _noalloc(lib, A, b):
    n = A.shape[0]
    Lm = np.zeros((n, n))
    x = np.zeros(n)
    st = lib.zs_dense_cholesky_solve_noalloc(_ptr(A), n, _ptr(b), _ptr(Lm), _ptr(x))
    return st, Lm, x


def _spd(n, seed):
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(n, n))
    return G @ G.T / n + np.eye(n), rng.normal(size=n)


def test_noalloc_matches_allocating_solve_twice(zs_lib):
    from zeroslam_gb300 import ba

    limit = 384  # ZS_NOALLOC_MAX_N
    for n, seed in ((limit, 1), (150, 2)):  # the second call reuses the workspace at a smaller n
        A, b = _spd(n, seed)
        ok, L_ref, x_ref = ba.dense_cholesky_solve(A, b)
        assert ok
        st, Lm, x = _noalloc(zs_lib, A, b)
        assert st == ba.ZS_OK
        assert rel_err(x, x_ref) < 1e-12
        assert rel_err(Lm, L_ref) < 1e-12


def test_noalloc_limits_and_failure(zs_lib):
    from zeroslam_gb300 import ba

    A, b = _spd(385, 3)
    st, _, _ = _noalloc(zs_lib, A, b)
    assert st == ba.ZS_ERR_INVALID  # beyond the fixed workspace
    A, b = _spd(64, 4)
    A[40, 40] = -1.0
    st, _, _ = _noalloc(zs_lib, A, b)
    assert st == ba.ZS_ERR_CHOLESKY
    A, b = _spd(64, 5)  # a failed call leaves nothing behind that the next one sees
    st, _, x = _noalloc(zs_lib, A, b)
    assert st == ba.ZS_OK and rel_err(x, np.linalg.solve(A, b)) < 1e-11
