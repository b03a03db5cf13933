// FP64 contractions of the plain form on the FP64 tensor path (DMMA).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cutc {

// C[m + ldc n] = alpha sum_k opA(m, k) B[n ldb + k] + beta C[m + ldc n]
// for m < M, n < N, over `batch` problems whose A, B and C start sa, sb and sc
// doubles apart.  opA(m, k) = A[m lda + k] when a_kmajor (K contiguous, cuBLAS
// OP_T on a K x M column-major array), else A[k lda + m] (M contiguous, OP_N).
// B is K contiguous per column n (OP_N on a K x N column-major array).  With
// beta == 0, C is not read.  Column-major C, as cuBLAS: the same call sites
// keep their argument meaning.
int fp64_gemm(cudaStream_t st, bool a_kmajor, int M, int N, int64_t K, double alpha,
              const double *A, int64_t lda, int64_t sa, const double *B, int64_t ldb, int64_t sb,
              double beta, double *C, int64_t ldc, int64_t sc, int batch);

}  // namespace cutc
