"""The tensor-core product of the mixed form's dense preconditioner
(tcgen05.mma kind::tf32 fed by TMA, three TF32 products per operand pair):
C = A B^T to FP32 accuracy against an FP64 product, on whole and partial
128 x 128 tiles, K not a multiple of the 32-wide K step, the
lower-triangle mode, and capped grids whose CTAs walk several tiles (the
ring of stages, the promoted chunks and the tensor memory carried from
tile to tile). Its error is held to twice that of numpy's own FP32
product of the same operands (plus a floor for tiny errors)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 128, 32), (1, 1, 4), (300, 200, 100), (129, 257, 36), (1024, 768, 1024),
                                   (640, 640, 3000)])
def test_tc_gemm_accuracy(zs_lib, M, N, K):
    from zeroslam_gb300 import ba

    rng = np.random.default_rng(M * 7 + N * 13 + K)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(N, K)).astype(np.float32)
    C, ms = ba.dense_gemm_tf32x3(A, B)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    err = np.max(np.abs(C - ref))
    err32 = np.max(np.abs(A @ B.T - ref))
    assert err <= 2.0 * err32 + 1e-6 * np.max(np.abs(ref)), (err, err32)
    assert ms > 0


def test_tc_gemm_lower(zs_lib):
    from zeroslam_gb300 import ba

    rng = np.random.default_rng(5)
    A = rng.normal(size=(400, 96)).astype(np.float32)
    C, _ = ba.dense_gemm_tf32x3(A, A, lower=True)
    ref = A.astype(np.float64) @ A.astype(np.float64).T
    low = np.tril(np.ones((400, 400), bool))
    assert np.all(C[~low] == 0.0)  # the upper triangle is left as it was (zero)
    assert np.max(np.abs(C[low] - ref[low])) <= 2.0 * np.max(np.abs((A @ A.T)[low] - ref[low])) + 1e-6 * 96


@pytest.mark.parametrize("M,N,K,cap,lower", [(1024, 768, 1024, 7, False), (300, 200, 100, 2, False),
                                             (129, 257, 36, 1, False), (640, 640, 3000, 5, False),
                                             (700, 700, 256, 3, True), (900, 300, 96, 4, True)])
def test_tc_gemm_capped_grid(zs_lib, M, N, K, cap, lower):
    from zeroslam_gb300 import ba

    rng = np.random.default_rng(M + 3 * N + 5 * K + cap)
    A = rng.normal(size=(M, K)).astype(np.float32)
    B = rng.normal(size=(N, K)).astype(np.float32)
    C, _ = ba.dense_gemm_tf32x3(A, B, lower=lower, max_ctas=cap)
    ref = A.astype(np.float64) @ B.astype(np.float64).T
    ref32 = A @ B.T
    mask = np.tril(np.ones((M, N), bool)) if lower else np.ones((M, N), bool)
    assert np.all(C[~mask] == 0.0)
    err = np.max(np.abs(C[mask] - ref[mask]))
    err32 = np.max(np.abs(ref32[mask] - ref[mask]))
    assert err <= 2.0 * err32 + 1e-6 * np.max(np.abs(ref)), (err, err32)
    full, _ = ba.dense_gemm_tf32x3(A, B, lower=lower)
    assert np.array_equal(C, full)  # the same sums whichever CTA takes a tile


def test_tc_gemm_lower_needs_tall(zs_lib):
    from zeroslam_gb300 import ba

    A = np.ones((100, 8), np.float32)
    B = np.ones((200, 8), np.float32)
    with pytest.raises(ba.ZsError):
        ba.dense_gemm_tf32x3(A, B, lower=True)
