"""The mixed form's FP32 preconditioner alone (zs_dense_chol_inverse_f32):
the factor S = L L^T of matrix::decompose_cholesky
(source/matrix_decomposition_cholesky.hpp:26-61) restated in FP32, and
X = L^-1, from the dataflow kernel (64 x 64 tiles, any n) and from the
blocked tensor-core form (panels of 256 columns, n % 4 == 0; the solves
take it from n = 3072 on),
against numpy's FP64 factor.

Tolerances: S is rounded to FP32 once (2^-24 relative) and the FP32 factor
adds rounding growing like sqrt(n) u; the test matrices have condition
numbers below 10, so L agrees with the FP64 factor to ~1e-5 relative (1e-4
is asserted) and X L = I to the same order. The two forms sum in different
orders and agree with each other at that level, not bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spd(n, seed, shift=1.0):
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(n, n))
    return G @ G.T / n + shift * np.eye(n)


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _check(A, L, X, tol=1e-4):
    n = A.shape[0]
    Lr = np.linalg.cholesky(A)
    L64 = L.astype(np.float64)
    X64 = X.astype(np.float64)
    assert _rel(L64, Lr) < tol
    assert np.linalg.norm(X64 @ L64 - np.eye(n)) / np.sqrt(n) < tol
    assert not np.triu(L64, 1).any() and not np.triu(X64, 1).any()


@pytest.mark.parametrize("n", [1, 63, 200, 640])
def test_dataflow_small(zs_lib, n):
    from zeroslam_gb300 import ba

    A = _spd(n, n)
    st, L, X, _ = ba.dense_chol_inverse_f32(A, form=1)
    assert st == ba.ZS_OK
    _check(A, L, X)


@pytest.mark.parametrize("n", [2048, 2100, 2560])
def test_blocked_matches_numpy(zs_lib, n):
    """Panels of 256 with a ragged last panel (2100 = 8 x 256 + 52) and the
    dataflow kernel's answer on the same matrix."""
    from zeroslam_gb300 import ba

    A = _spd(n, n)
    st, L, X, _ = ba.dense_chol_inverse_f32(A, form=2)
    assert st == ba.ZS_OK
    _check(A, L, X)
    st1, L1, X1, _ = ba.dense_chol_inverse_f32(A, form=1)
    assert st1 == ba.ZS_OK
    assert _rel(L.astype(np.float64), L1.astype(np.float64)) < 1e-4
    assert _rel(X.astype(np.float64), X1.astype(np.float64)) < 1e-4


def test_solve_form_3600(zs_lib):
    """The form the solves choose at n = 3600: blocked (n >= 3072), 14 panels
    of 256 and a last panel of 16 columns (a dataflow launch of one tile, the
    products with K = 16)."""
    from zeroslam_gb300 import ba

    A = _spd(3600, 3600)
    st, L, X, _ = ba.dense_chol_inverse_f32(A, form=0)
    assert st == ba.ZS_OK
    _check(A, L, X)


def test_blocked_6000(zs_lib):
    """The size of the loop workload's reduced camera system: 24 panels."""
    from zeroslam_gb300 import ba

    A = _spd(6000, 6000)
    st, L, X, ms = ba.dense_chol_inverse_f32(A, form=0)
    assert st == ba.ZS_OK and ms > 0.0
    _check(A, L, X)


def test_blocked_form_rules(zs_lib):
    from zeroslam_gb300 import ba

    with pytest.raises(ba.ZsError):
        ba.dense_chol_inverse_f32(_spd(2050, 1), form=2)  # n % 4 != 0
    st, L, X, _ = ba.dense_chol_inverse_f32(_spd(3074, 2), form=0)  # the dataflow kernel serves it
    assert st == ba.ZS_OK
    _check(_spd(3074, 2), L, X)
    A = _spd(300, 3)  # two panels, the second 44 wide
    st, L, X, _ = ba.dense_chol_inverse_f32(A, form=2)
    assert st == ba.ZS_OK
    _check(A, L, X)


@pytest.mark.parametrize("n,form", [(200, 1), (640, 1), (1024, 2), (2100, 2)])
def test_reads_lower_triangle_only(zs_lib, n, form):
    """matrix::decompose_cholesky reads only S's lower triangle
    (source/matrix_decomposition_cholesky.hpp:42-50); so do both forms (the
    blocked form's trailing updates write only the lower triangle of the
    diagonal blocks the dataflow kernel then factors). Garbage above the
    diagonal leaves the factor and inverse unchanged."""
    from zeroslam_gb300 import ba

    A = _spd(n, n + 7)
    rng = np.random.default_rng(n)
    B = np.tril(A) + np.triu(3.0 + rng.random((n, n)), 1)
    st, L, X, _ = ba.dense_chol_inverse_f32(B, form=form)
    assert st == ba.ZS_OK
    _check(A, L, X)


@pytest.mark.parametrize("form", [1, 2])
def test_indefinite_fails(zs_lib, form):
    """A matrix with negative eigenvalues fails a pivot in some panel: the
    status is ZS_ERR_CHOLESKY and every later launch returns at once."""
    from zeroslam_gb300 import ba

    A = _spd(2100, 5, shift=-0.5)  # eigenvalues of G G^T / n span [0, 4]
    st, _, _, _ = ba.dense_chol_inverse_f32(A, form=form)
    assert st == ba.ZS_ERR_CHOLESKY
