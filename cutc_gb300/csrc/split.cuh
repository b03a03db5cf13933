// Split-precision (BF16-slice) contractions: plan and entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.cuh"
#include "pair.cuh"

namespace cutc {

constexpr int kMaxSlices = 7;
constexpr int kDefaultSlices = 5;

// One FP64 operand as S BF16 slices [S][Mpad][Kpad] plus row exponents.
struct Operand {
    void *sl = nullptr;               // __nv_bfloat16 slices
    int *ex = nullptr;                // row exponents (Mpad)
    unsigned long long *rmax = nullptr;
    int M = 0, Mpad = 0;
    int64_t K = 0, Kpad = 0;
};

struct SplitPlan {
    int slot0 = 0;
    int n_slices = 0;
    int64_t n1t = 0;
    Operand AX;                        // P slices: X-build A operand
    Operand BX;                        // G-tile slices: X-build B operand
    // pair terms on the tensor cores: F slices (powers of f2 on r2), the tile's
    // coefficient slices, and their FP64 sources
    bool pair_tc = false;
    int pair_slices = 5;
    Operand AF, BC;
    double *Fd = nullptr, *Cd = nullptr;
    float2 *r1d = nullptr;             // the tile's r1 points in double-float
    float *bscale = nullptr;           // 2^(row exponent) of the coefficient rows
    int2 *pairs_sym = nullptr;         // (a, b), a >= b, in tri_index order
    int2 *pairs_anti = nullptr;        // (a, b), a > b, in stri_index order
    int *err = nullptr;                // device flag set by a bounded wait that gave up
};

// Device bytes per r1 row of an X tile (slices of G).
size_t split_r1_row_bytes(const Request &R);
// 32-wide K blocks per tensor-core launch of a contraction over K with an A operand of
// M rows (k_split as in cutc_options: 0 = one launch up to K = 65536, equal launches of
// <= 49152 beyond; for M >= 16384 one launch up to 32768, launches of <= 24576 beyond).
int split_k_blocks_per_launch(int64_t K, int64_t M, int k_split);
// Device bytes per r1 row of an int_2e block (slices of its int_2e operands).
size_t split_int2e_row_bytes(const Request &R);
// Device bytes that do not depend on the tile size (the P slices).
size_t split_fixed_bytes(const Request &R);
// The bounded-wait check behind cutc_check_wait_limit: CUTC_ERR_TIMEOUT when the
// wait gave up as designed.
int split_wait_limit_check(Engine *E);
int split_prepare_x(Engine *E, const Request &R, cudaStream_t st, const double *wr2,
                    const double *aos2v, int64_t n1t, int slot0, SplitPlan &sp);
// X of one r1 tile from the df tile G[c][i][j] ((hi, lo) pairs), written into the
// int_2e block buffer Xb[(m blk_rows + ib + i) np + p] (the tile starts at row ib of
// a block of blk_rows rows).  have_rmax: the row maxima of G are already in
// sp.BX.rmax (rows c nb + i).
int split_x_tile(Engine *E, const Request &R, cudaStream_t st, SplitPlan &sp, const float2 *G,
                 int nb, double *Xb, int blk_rows, int ib, cudaEvent_t gemm_begin,
                 cudaEvent_t gemm_end, bool have_rmax = false);
// Adds an r1 block's share of the int_2e contractions to H and N (overwrites when
// first): wr1 and aos1 point at the block's first row, ld1 is the row stride of aos1,
// Xt[(m nb + i) np + p] holds the block's X rows.
int split_int2e_tile(Engine *E, const Request &R, cudaStream_t st, SplitPlan &sp,
                     const double *wr1, const double *aos1, int64_t ld1, int nb, const double *Xt,
                     double *H, double *N, bool first);
// The pair terms of a split-form build on the tensor cores: applicable when every
// Jastrow exponent is 0, 2, 3 or 4, n_nuc <= 20, the build uses 5 slices and neither
// FP64 pair terms nor CUTC_PAIR_DF / CUTC_PAIR_DENSE (the double-float kernels) is asked
// for.
bool split_pair_tc_ok(const Request &R, const int *exps, int n_terms);
// Builds the F operand (powers of f2 on the r2 points; f2 is [n_nuc][n2] FP64) once per
// build and reserves the coefficient operand for tiles of up to n1t rows.
int split_pair_prepare(Engine *E, const Request &R, cudaStream_t st, const double *f2,
                       int64_t n1t, SplitPlan &sp);
// The pair planes G of one r1 tile (P: the tile's rows, outputs and near-coalescence
// data, as for launch_pair_df; its rmax must be zeroed).
int split_pair_tile(Engine *E, const Request &R, cudaStream_t st, SplitPlan &sp,
                    const PairDfArgs &P, const double *rn, double a_en);
// Device bytes of the tensor-core pair operands: fixed (F) and per r1 row of a tile.
size_t split_pair_fixed_bytes(const Request &R);
size_t split_pair_row_bytes(const Request &R);
// Reports a bounded wait that gave up in any of the launches (synchronises).
int split_check(cudaStream_t st, SplitPlan &sp);
// C[m + ldc n] = sum_k A[m K + k] B[n K + k] through the split form (device arrays)
int split_gemm_dense(Engine *E, cudaStream_t st, int n_slices, int M, int N, int64_t K,
                     const double *A, const double *B, double *C, int64_t ldc);
// C[m + ldc n] = alpha (A1[m K1 + k] B1[n K1 + k] summed over k < K1 + A2 B2^T likewise
// over K2), as one split contraction over the concatenated K (device arrays)
int split_gemm_concat(Engine *E, cudaStream_t st, int n_slices, int M, int N, int64_t K1,
                      const double *A1, const double *B1, int64_t K2, const double *A2,
                      const double *B2, double alpha, double *C, int64_t ldc);

}  // namespace cutc
