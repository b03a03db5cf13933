"""The tcgen05 split-precision GEMM against an FP64 reference.

Each operand row is cut into S signed 9-bit BF16 slices of its own scale
(rounding error <= 2^-(9S) of the row maximum), so element (m, n) of the
product is bounded by

    |C - AB^T|_mn <= tol(S) * (max|A_m| |B_n|_1 + |A_m|_1 max|B_n|)

with tol(S) = max(2^-(9S-3), 2^-50): the slice diagonals 0, 1 and 2 are
accumulated exactly across the 128-wide K chunks (diagonal 2 can round only when
its remainder digits add up coherently over a chunk, which random operands never
do), and the remaining diagonals (relative size 2^-27 and below) in FP32, so no
error term grows with K beyond the FP64 recombination.
"""
import numpy as np
import pytest

import cutc_gb300 as cg

pytestmark = pytest.mark.gpu


def _ref(A, B):
    return A @ B.T, np.abs(A) @ np.abs(B).T


def _bound(A, B, S):
    K = A.shape[1]
    tol = max(2.0 ** -(9 * S - 3), 2.0 ** -50)
    a_inf, b_inf = np.abs(A).max(axis=1), np.abs(B).max(axis=1)
    a_1, b_1 = np.abs(A).sum(axis=1), np.abs(B).sum(axis=1)
    return tol * (a_inf[:, None] * b_1[None, :] + a_1[:, None] * b_inf[None, :])


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (130, 70, 100), (300, 257, 1000),
                                   (7, 5, 3), (1000, 200, 5000)])
@pytest.mark.parametrize("S", [5])
def test_split_gemm_random(M, N, K, S):
    import torch
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-5, 5, size=(M, 1)))
    B = rng.standard_normal((N, K)) * np.exp(rng.uniform(-5, 5, size=(N, 1)))
    C = cg.split_gemm_device(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), n_slices=S)
    C = C.cpu().numpy()
    R, Ab = _ref(A, B)
    assert np.all(np.abs(C - R) <= _bound(A, B, S)), (np.abs(C - R) / _bound(A, B, S)).max()
    # and in the usual dot-product scale
    assert (np.abs(C - R) / Ab).max() < 2.0 ** -38


@pytest.mark.parametrize("S", [3, 4, 6, 7])
def test_split_gemm_slice_counts(S):
    import torch
    rng = np.random.default_rng(S)
    M, N, K = 200, 100, 700
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((N, K))
    C = cg.split_gemm_device(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), n_slices=S)
    R, Ab = _ref(A, B)
    C = C.cpu().numpy()
    assert np.all(np.abs(C - R) <= _bound(A, B, S)), (np.abs(C - R) / _bound(A, B, S)).max()


def test_split_gemm_wide_dynamic_range_and_zeros():
    """Rows spanning 2^-60..2^60, an all-zero row, exact zeros inside rows."""
    import torch
    rng = np.random.default_rng(3)
    M, N, K = 150, 90, 2000
    A = rng.standard_normal((M, K)) * np.exp2(rng.uniform(-60, 60, size=(M, K)))
    B = rng.standard_normal((N, K))
    A[5] = 0.0
    B[:, ::7] = 0.0
    C = cg.split_gemm_device(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), n_slices=5)
    R, Ab = _ref(A, B)
    C = C.cpu().numpy()
    assert np.all(C[5] == 0.0)
    # per element, against max|A_m| |B_n|_1 (tiny entries fall below the slices)
    bound = np.abs(A).max(axis=1)[:, None] * np.abs(B).sum(axis=1)[None, :]
    assert np.all(np.abs(C - R) <= 2.0 ** -40 * bound + 1e-300)


def test_split_gemm_long_k_exact_accumulation():
    """K = 2^17: exactness of the chunked accumulation keeps the error at the slice level."""
    import torch
    rng = np.random.default_rng(11)
    M, N, K = 128, 64, 1 << 17
    A = np.abs(rng.standard_normal((M, K)))  # same signs: worst case for accumulation
    B = np.abs(rng.standard_normal((N, K)))
    C = cg.split_gemm_device(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), n_slices=5)
    R, Ab = _ref(A, B)
    C = C.cpu().numpy()
    assert np.all(np.abs(C - R) <= _bound(A, B, 5))
    assert (np.abs(C - R) / Ab).max() < 2.0 ** -40


def test_split_gemm_extreme_row_scales():
    """Row scales 2^-540 .. 2^500 on both sides: products from 2^-1080 (subnormal or zero
    results) to 2^1000 (near the top of the FP64 range), with the sign of each."""
    import torch
    rng = np.random.default_rng(17)
    M, N, K = 140, 60, 300
    ea = rng.choice([-540, -300, 0, 300, 500], size=(M, 1))
    eb = rng.choice([-540, -300, 0, 300, 500], size=(N, 1))
    A = rng.standard_normal((M, K)) * np.exp2(ea.astype(float))
    B = rng.standard_normal((N, K)) * np.exp2(eb.astype(float))
    C = cg.split_gemm_device(torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda(), n_slices=5)
    C = C.cpu().numpy()
    R, _ = _ref(A, B)
    assert np.all(np.isfinite(C))
    # the slice bound, plus K units of the smallest subnormal: numpy's own products round
    # to subnormals where they underflow
    assert np.all(np.abs(C - R) <= _bound(A, B, 5) + 2 * K * 2.0 ** -1074)
    big = (ea + eb.T) >= 0
    assert np.all(np.sign(C[big]) == np.sign(R[big]))
