"""The plain form's FP64 DMMA GEMM (cutc_fp64_gemm_dev) against numpy FP64.

The kernel replaces the reference's cublasDgemm calls
(src/build_int2_grad1_u12_ao.cu:152-159, src/build_int_2e_ao.cu:60-67,97-104)
with cuBLAS's column-major argument meaning.  Each case checks every element
against numpy within 1e-13 of sum_k |opA(m, k) B(k, n)| (a different summation
order is the only difference), plus alpha, beta, leading dimensions larger
than the extents, batch strides, ragged tile edges and K = 0.
"""
import numpy as np
import pytest

import cutc_gb300 as cg

pytestmark = pytest.mark.gpu


def _case(a_kmajor, M, N, K, lda, ldb, ldc, alpha, beta, batch=1, seed=0):
    import torch
    rng = np.random.default_rng(seed)
    # each operand as a row-major host array, with padding columns of NaN that must not be read
    a_rows, a_cols = (M, lda) if a_kmajor else (K, lda)
    A = rng.standard_normal((batch, a_rows, a_cols))
    B = rng.standard_normal((batch, N, ldb))
    C0 = rng.standard_normal((batch, N, ldc))
    if a_kmajor:
        A[:, :, K:] = np.nan
    else:
        A[:, :, M:] = np.nan
    B[:, :, K:] = np.nan
    C0[:, :, M:] = 7.0  # outside the M rows: must stay as is
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(B).cuda()
    dC = torch.from_numpy(C0.copy()).cuda()
    cg.fp64_gemm_device(a_kmajor, M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc,
                        stride_a=a_rows * a_cols, stride_b=N * ldb, stride_c=N * ldc, batch=batch)
    got = dC.cpu().numpy()
    for z in range(batch):
        opA = A[z, :, :K] if a_kmajor else A[z, :K, :M].T   # M x K
        Bk = B[z, :, :K]                                    # N x K
        ref = alpha * opA @ Bk.T + (beta * C0[z, :, :M].T if beta != 0 else 0.0)  # M x N
        bound = abs(alpha) * np.abs(opA) @ np.abs(Bk).T + (abs(beta) * np.abs(C0[z, :, :M].T))
        err = np.abs(got[z, :, :M].T - ref)
        assert np.all(err <= 1e-13 * bound + 1e-300), (z, float(np.max(err / (bound + 1e-300))))
        assert np.all(got[z, :, M:] == 7.0)


@pytest.mark.parametrize("a_kmajor", [True, False])
def test_fp64_gemm_shapes(a_kmajor):
    _case(a_kmajor, 130, 129, 35, 140, 37, 131, 1.0, 0.0)         # ragged M, N, K edges
    _case(a_kmajor, 1, 1, 1, 3, 1, 1, 2.5, 0.0)                   # one element
    _case(a_kmajor, 300, 257, 1000, 1003, 1001, 301, -0.5, 1.0)   # beta = 1 accumulation
    _case(a_kmajor, 64, 200, 17, 70, 19, 64, 1.0, 0.25, batch=3)  # batched, strided


def test_fp64_gemm_k_zero_scales_c():
    _case(True, 40, 30, 0, 1, 1, 41, 1.0, 2.0)


def test_fp64_gemm_rejects_bad_leading_dimensions():
    import torch
    A = torch.zeros((8, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(cg.CutcError) as e:
        cg.fp64_gemm_device(True, 8, 8, 8, 1.0, A, 4, A, 8, 0.0, A, 8)  # lda < K
    assert e.value.status == cg.CUTC_ERR_INVALID
