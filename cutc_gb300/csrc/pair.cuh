// Pair-term (grad1 u) kernels: argument block and launchers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cutc {

// (f, d f/dx, d f/dy, d f/dz) of one (point, nucleus) pair
struct __align__(32) NucTerm {
    double f, gx, gy, gz;
};

struct PairArgs {
    int i0;            // first r1 row of the tile (global index)
    int n1b;           // r1 rows in the tile
    int n2;            // r2 points
    int nN;            // nuclei
    int n_terms;       // Jastrow terms kept (|c| >= 1e-10)
    const double *r1;  // (3, n_grid1) AoS
    const double *r2;  // (3, n2) AoS
    const NucTerm *t1; // [n1b][nN] (f1, grad f1) of the tile's rows
    const double *f2;  // [nN][n2]
    const double *coef;     // [n_terms][3] = (c m, c n, c o)
    const int *exps;        // [n_terms] = m | n << 3 | o << 6
    const int *term_off;    // [nN + 1] first term of each nucleus
    double a_ee;
    double *G;         // G[c * plane + i * ldg + j]
    int64_t ldg;
    int64_t plane;
};

// r12^2 below which the split form's pair kernels take the coordinate differences in
// FP64 (where they are exact) instead of double-float.
constexpr float kNearPairR2 = 1.0e-4f;

// The high word of the FP64 form of a non-negative float given by its bits (float
// subnormals count as 2^-126): the row-maximum word the slicers read.  It is a
// non-decreasing function of the bits, so the maximum of a warp's words is the word of
// the warp's largest bits, and one conversion after the reduction serves the warp.
__device__ __forceinline__ unsigned rmax_word(unsigned fb)
{
    const unsigned ef = fb >> 23;
    return fb == 0u ? 0u : ef == 0u ? (897u << 20) : ((ef + 896u) << 20) | ((fb & 0x7fffffu) >> 3);
}

// Arguments of the double-float pair kernel (split form).
struct PairDfArgs {
    int i0, n1b, n2, nN;
    int rows_per_cta;       // set by the launcher
    const double *r1;       // (3, n_grid1) AoS, FP64
    const double *r2;       // (3, n2) AoS, FP64 (near-coalescence path)
    const float2 *r2d;      // [3][n2] df coordinates
    const double *f2;       // [nN][n2] FP64 (near-coalescence path)
    const float2 *f2d;      // [nN][n2] df
    const NucTerm *t1;      // [n1b][nN] FP64 per-point terms (near-coalescence path)
    const float2 *poly;     // [n1b][nN][kN] df polynomial coefficients (written by the launcher)
    float2 *poly_w;
    const double *coef;     // term table, as PairArgs
    const int *exps;
    const int *term_off;
    double a_ee;            // FP64 (near path)
    float a_ee_hi, a_ee_lo; // df
    float2 *G;              // G[c * plane + i * ldg + j] as (hi, lo)
    int64_t ldg;
    int64_t plane;
    // optional: rmax[c * n1b + i] |= bits of max_j |G| (only its exponent field is
    // exact: it is the max of the high 32 bits), for the split slicer
    unsigned long long *rmax = nullptr;
};

int pair_df_max_exp(const int *exps, int n_terms);
// True when every exponent of the term table is 0, 2, 3 or 4 (the sparse-power kernel applies).
bool pair_df_sparse(const int *exps, int n_terms);
// in place: x[i] (FP64) -> (hi, lo) float pair at the same 8 bytes
int launch_f64_to_df(cudaStream_t st, double *x, int64_t n);
size_t pair_df_poly_bytes(int E, int n1b, int nN);
int launch_r2_df(cudaStream_t st, int n2, int nN, const double *r2, const double *f2, float2 *r2d,
                 float2 *f2d);
int launch_pair_df(cudaStream_t st, const PairDfArgs &P, int E, bool sparse, const double *rn,
                   double a_en);

// Operands of the tensor-core pair terms (exponents in {0, 2, 3, 4}), FP64: the powers
// F[j * 4 nN + 4 A + q] = f2_A(r2_j)^b_q (b = 0, 2, 3, 4) and, for r1 rows [i0, i0 + n),
// the 16 coefficient rows C[((i 16 + c) 4 nN) + 4 A + q] of each point, with the points
// themselves in double-float, r1d[3 i + c].
int launch_pair_tc_f(cudaStream_t st, int n2, int nN, const double *f2, double *F);
int launch_pair_tc_coef(cudaStream_t st, int i0, int n, int nN, const double *r1, const double *rn,
                        double a_en, const double *coef, const int *exps, const int *term_off,
                        double *C, float2 *r1d);

int launch_r1_terms(cudaStream_t st, int i0, int n, int nN, const double *r1, const double *rn,
                    double a, NucTerm *t1);
int launch_r2_terms(cudaStream_t st, int n2, int nN, const double *r2, const double *rn,
                    double a, double *f2);
int launch_pair_f64(cudaStream_t st, const PairArgs &P);

}  // namespace cutc
