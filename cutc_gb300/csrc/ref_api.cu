// The reference's device-level entry points of the cutc_int path, under its
// names and signatures, for callers that drive the stages themselves:
//
//   cutc_int_bh              src/jast_bh.cu:268-303
//   int_long_range           src/long_range_integ.cu:52-67
//   int_short_range_herm     src/short_range_integ_herm.cu:51-64
//   int_short_range_nonherm  src/short_range_integ_nonherm.cu:69-82
//   get_int2_grad1_u12_ao    src/build_int2_grad1_u12_ao.cu:9-347
//   get_int_2e_ao            src/build_int_2e_ao.cu:11-145
//
// As in the reference, every array is a device pointer and the work is ordered
// on the legacy default stream, so it follows the caller's own default-stream
// work; the reference signatures return nothing, so failures are recorded for
// cutc_last_error() instead of ending the process.  The launch geometry the
// reference takes for its pair kernel is validated like cutc_int's and then
// ignored.  What runs is this library's:
//   * the product kernels write the reference's full nA^2 layouts, one thread
//     per (grid point, first AO) walking the second AO, so every store of a
//     warp is 32 consecutive doubles (the reference: one thread per point
//     writing nA^2 values at stride n);
//   * cutc_int_bh is the FP64 pair kernel of the plain form, on the r2 window
//     and strides the reference's layout asks for;
//   * get_int2_grad1_u12_ao is the streamed X build of cutc_int_ex (r1 tiles,
//     packed AO pairs; plain FP64 unless CUTC_PRECISION=split, with CUTC_SLICES
//     slices) without int_2e;
//   * get_int_2e_ao contracts the caller's full X (it need not be symmetric in
//     the AO pair) against the short-range products in r1 blocks sized to a
//     byte budget, with the FP64 DMMA GEMM accumulating in FP64, then adds A^T.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "dgemm.cuh"
#include "engine.cuh"

namespace cutc {

// out[g + ld_out (j + nA i)] = (w[g] chi_i(g)) chi_j(g) for g < n, i, j < nA, where
// chi_a(g) = chi[a * ld_chi + g]  (src/long_range_integ.cu:39,
// src/short_range_integ_herm.cu:38: the same products in the same order)
__global__ void full_sym_products_kernel(int n, int nA, const double *__restrict__ w,
                                         const double *__restrict__ chi, int64_t ld_chi,
                                         double *__restrict__ out, int64_t ld_out)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (g >= n)
        return;
    const double wi = w[g] * chi[(int64_t)i * ld_chi + g];
    double *o = out + (int64_t)nA * i * ld_out + g;
    for (int j = 0; j < nA; j++)
        o[(int64_t)j * ld_out] = wi * chi[(int64_t)j * ld_chi + g];
}

// out[g + ldm m + ldp (j + nA i)] = w (chi_j d_m chi_i - chi_i d_m chi_j), m < 3
// (src/short_range_integ_nonherm.cu:55); component k of AO a at
// aos[(k nA + a) ld_aos + g], k = 0 the value, k = 1..3 the gradient.
__global__ void full_antisym_products_kernel(int n, int nA, const double *__restrict__ w,
                                             const double *__restrict__ aos, int64_t ld_aos,
                                             double *__restrict__ out, int64_t ldm, int64_t ldp)
{
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (g >= n)
        return;
    const int64_t comp = (int64_t)nA * ld_aos;
    const double wg = w[g];
    const double vi = aos[(int64_t)i * ld_aos + g];
    const double di[3] = {aos[comp + (int64_t)i * ld_aos + g],
                          aos[2 * comp + (int64_t)i * ld_aos + g],
                          aos[3 * comp + (int64_t)i * ld_aos + g]};
    double *o = out + (int64_t)nA * i * ldp + g;
    for (int j = 0; j < nA; j++) {
        const double vj = aos[(int64_t)j * ld_aos + g];
#pragma unroll
        for (int m = 0; m < 3; m++) {
            const double dj = aos[(m + 1) * comp + (int64_t)j * ld_aos + g];
            o[(int64_t)j * ldp + m * ldm] = wg * (vj * di[m] - vi * dj);
        }
    }
}

static int launch_full_sym(cudaStream_t st, int n, int nA, const double *w, const double *chi,
                           int64_t ld_chi, double *out, int64_t ld_out)
{
    if (n <= 0)
        return CUTC_OK;
    dim3 grid(ceil_div(n, 128), nA);
    full_sym_products_kernel<<<grid, 128, 0, st>>>(n, nA, w, chi, ld_chi, out, ld_out);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    return CUTC_OK;
}

static int launch_full_antisym(cudaStream_t st, int n, int nA, const double *w, const double *aos,
                               int64_t ld_aos, double *out, int64_t ldm, int64_t ldp)
{
    if (n <= 0)
        return CUTC_OK;
    dim3 grid(ceil_div(n, 128), nA);
    full_antisym_products_kernel<<<grid, 128, 0, st>>>(n, nA, w, aos, ld_aos, out, ldm, ldp);
    CUTC_CUDA_TRY(cudaGetLastError());
    note_launches(1);
    return CUTC_OK;
}

static bool ao_count_ok(const char *what, int n_ao)
{
    if (n_ao <= 0 || n_ao > 65535 || (int64_t)n_ao * n_ao > (int64_t)INT32_MAX / 2) {
        cutc_set_error(CUTC_ERR_INVALID, "%s: n_ao = %d out of range", what, n_ao);
        return false;
    }
    return true;
}

// Slots of the engine workspace used here (the build's own slots are below 180).
enum RefSlot { R_S0 = 200, R_S };

// int_2e = A + A^T with A = X_3 S0 - 1/2 sum_m X_m S_m over all n1 r1 points,
// X (nA^2, n1, 4) the caller's full array; r1 blocks of K rows, FP64 accumulation.
static int int2e_from_full_x(Engine *E, cudaStream_t st, int n1, int nA, const double *w1,
                             const double *aos1, const double *X, double *I)
{
    const int64_t nA2 = (int64_t)nA * nA;
    size_t free_b = 0, total_b = 0;
    CUTC_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    size_t budget = std::min<size_t>((size_t)16 << 30, free_b / 4);
    if (const char *e = getenv("CUTC_INT2E_ROWS"))  // cap, for tests of the blocking
        budget = std::min<size_t>(budget, (size_t)std::max(1, atoi(e)) * 32 * nA2);
    const int K = (int)std::max<int64_t>(1, std::min<int64_t>(n1, budget / (32 * nA2)));
    void *p;
    Workspace &W = E->ws;
    CUTC_TRY(W.get(R_S0, (size_t)K * nA2 * 8, &p));
    double *S0 = (double *)p;
    CUTC_TRY(W.get(R_S, 3 * (size_t)K * nA2 * 8, &p));
    double *S = (double *)p;
    const double one = 1.0, mhalf = -0.5;
    for (int g0 = 0; g0 < n1; g0 += K) {
        const int Kb = std::min(K, n1 - g0);
        // S0[g + Kb q], S[g + Kb m + 3 Kb q] for the block's points
        CUTC_TRY(launch_full_sym(st, Kb, nA, w1 + g0, aos1 + g0, n1, S0, Kb));
        CUTC_TRY(launch_full_antisym(st, Kb, nA, w1 + g0, aos1 + g0, n1, S, Kb, 3 * (int64_t)Kb));
        const double beta0 = g0 == 0 ? 0.0 : 1.0;
        // I = X_3 S0 (+ I)   (src/build_int_2e_ao.cu:60-67)
        CUTC_TRY(fp64_gemm(st, false, (int)nA2, (int)nA2, Kb, one,
                           X + nA2 * (3 * (int64_t)n1 + g0), nA2, 0, S0, Kb, 0, beta0, I, nA2, 0,
                           1));
        // I += -1/2 X_m S_m   (src/build_int_2e_ao.cu:97-104, one product per component)
        for (int m = 0; m < 3; m++)
            CUTC_TRY(fp64_gemm(st, false, (int)nA2, (int)nA2, Kb, mhalf,
                               X + nA2 * ((int64_t)m * n1 + g0), nA2, 0, S + (int64_t)m * Kb,
                               3 * (int64_t)Kb, 0, one, I, nA2, 0, 1));
    }
    return CUTC_OK;
}

static void report(int status, const char *what)
{
    // the status itself is already recorded; a CUDA error left by a launch is not
    const cudaError_t e = cudaGetLastError();
    if (status == CUTC_OK && e != cudaSuccess)
        cutc_set_error(CUTC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

static int precision_from_env()
{
    const char *prec = getenv("CUTC_PRECISION");
    return (prec && strcmp(prec, "split") == 0) ? CUTC_SPLIT_BF16 : CUTC_PLAIN_FP64;
}

// CUTC_SLICES as cutc_int reads it: a malformed or out-of-range count is passed on
// for the build's own validation to refuse
static int slices_from_env(int fallback)
{
    const char *sl = getenv("CUTC_SLICES");
    if (!sl || !*sl)
        return fallback;
    char *end = nullptr;
    const long v = strtol(sl, &end, 10);
    return (*end == '\0' && v >= 0 && v <= 64) ? (int)v : -1;
}

}  // namespace cutc

using namespace cutc;

extern "C" void int_long_range(int jj0, int n_grid2_eff, int n_grid2_tot, int n_grid2, int n_ao,
                               double *wr2, double *aos_data2, double *int_fct_long_range)
{
    if (!ao_count_ok("int_long_range", n_ao))
        return;
    if (jj0 < 0 || n_grid2_eff < 0 || n_grid2_tot < n_grid2_eff || jj0 + n_grid2_eff > n_grid2 ||
        !wr2 || !aos_data2 || !int_fct_long_range) {
        cutc_set_error(CUTC_ERR_INVALID, "int_long_range: invalid arguments");
        return;
    }
    report(launch_full_sym(0, n_grid2_eff, n_ao, wr2 + jj0, aos_data2 + jj0, n_grid2,
                           int_fct_long_range, n_grid2_tot),
           "int_long_range");
}

extern "C" void int_short_range_herm(int n_grid1, int n_ao, double *wr1, double *aos_data1,
                                     double *int_fct_short_range_herm)
{
    if (!ao_count_ok("int_short_range_herm", n_ao))
        return;
    if (n_grid1 < 0 || !wr1 || !aos_data1 || !int_fct_short_range_herm) {
        cutc_set_error(CUTC_ERR_INVALID, "int_short_range_herm: invalid arguments");
        return;
    }
    report(launch_full_sym(0, n_grid1, n_ao, wr1, aos_data1, n_grid1, int_fct_short_range_herm,
                           n_grid1),
           "int_short_range_herm");
}

extern "C" void int_short_range_nonherm(int n_grid1, int n_ao, double *wr1, double *aos_data1,
                                        double *int_fct_short_range_nonherm)
{
    if (!ao_count_ok("int_short_range_nonherm", n_ao))
        return;
    if (n_grid1 < 0 || !wr1 || !aos_data1 || !int_fct_short_range_nonherm) {
        cutc_set_error(CUTC_ERR_INVALID, "int_short_range_nonherm: invalid arguments");
        return;
    }
    report(launch_full_antisym(0, n_grid1, n_ao, wr1, aos_data1, n_grid1,
                               int_fct_short_range_nonherm, n_grid1, 3 * (int64_t)n_grid1),
           "int_short_range_nonherm");
}

extern "C" void cutc_int_bh(cutc_dim3 dimGrid, cutc_dim3 dimBlock, int ii0, int n_grid1_eff,
                            int n_grid1_tot, int jj0, int n_grid2_eff, int n_grid2_tot, int n_nuc,
                            int size_bh, double *r1, double *r2, double *rn, double *c_bh,
                            int *m_bh, int *n_bh, int *o_bh, double *grad1_u12)
{
    if (cutc_validate_launch_dims((int)dimGrid.x, (int)dimGrid.y, (int)dimGrid.z, (int)dimBlock.x,
                                  (int)dimBlock.y, (int)dimBlock.z) != CUTC_OK)
        return;
    if (n_grid1_eff > n_grid1_tot || n_grid2_eff > n_grid2_tot) {
        cutc_set_error(CUTC_ERR_INVALID, "cutc_int_bh: effective sizes exceed the totals");
        return;
    }
    if (n_grid1_eff <= 0 || n_grid2_eff <= 0)
        return;  // nothing to write, as the reference's grid-stride loops
    Engine *E = nullptr;
    if (get_engine(&E) != CUTC_OK)
        return;
    std::lock_guard<std::mutex> lk(E->mu);
    // The reference fixes a_en = a_ee = 1 (src/jast_bh.cu:145,171,191).
    const int64_t ld = n_grid2_tot, plane = (int64_t)n_grid1_tot * n_grid2_tot;
    report(run_pair_only(E, cudaStreamLegacy, ii0, n_grid1_eff, ii0 + n_grid1_eff, jj0,
                         n_grid2_eff, ld, plane, n_nuc, size_bh, r1, r2, rn, c_bh, m_bh, n_bh,
                         o_bh, 1.0, 1.0, grad1_u12),
           "cutc_int_bh");
}

extern "C" void get_int2_grad1_u12_ao(cutc_dim3 dimGrid, cutc_dim3 dimBlock, int n_grid1,
                                      int n_grid2, int n_ao, int n_nuc, int size_bh, double *r1,
                                      double *r2, double *wr2, double *rn, double *aos_data2,
                                      double *c_bh, int *m_bh, int *n_bh, int *o_bh,
                                      double *int2_grad1_u12_ao)
{
    if (cutc_validate_launch_dims((int)dimGrid.x, (int)dimGrid.y, (int)dimGrid.z, (int)dimBlock.x,
                                  (int)dimBlock.y, (int)dimBlock.z) != CUTC_OK)
        return;
    Engine *E = nullptr;
    if (get_engine(&E) != CUTC_OK)
        return;
    Request R{};
    R.precision = precision_from_env();
    if (R.precision == CUTC_SPLIT_BF16)
        R.n_slices = slices_from_env(R.n_slices);
    R.x_components = 4;  // the reference's device array holds all four (m = 3: -1/2 |grad u|^2)
    R.device_pointers = 1;
    R.x_only = 1;
    R.stream = cudaStreamLegacy;
    R.n1 = n_grid1; R.n2 = n_grid2; R.nA = n_ao; R.nN = n_nuc; R.nB = size_bh;
    R.r1 = r1; R.r2 = r2; R.wr2 = wr2; R.rn = rn; R.aos2 = aos_data2;
    R.c_bh = c_bh; R.m_bh = m_bh; R.n_bh = n_bh; R.o_bh = o_bh;
    R.X = int2_grad1_u12_ao;
    std::lock_guard<std::mutex> lk(E->mu);
    const int s = run_build(E, R, nullptr);
    if (s != CUTC_OK)
        cudaStreamSynchronize(cudaStreamLegacy);
    report(s, "get_int2_grad1_u12_ao");
}

extern "C" void get_int_2e_ao(int n_grid1, int n_ao, double *wr1, double *aos_data1,
                              double *int2_grad1_u12, double *int_2e_ao)
{
    if (!ao_count_ok("get_int_2e_ao", n_ao))
        return;
    if (n_grid1 <= 0 || !wr1 || !aos_data1 || !int2_grad1_u12 || !int_2e_ao) {
        cutc_set_error(CUTC_ERR_INVALID, "get_int_2e_ao: invalid arguments");
        return;
    }
    Engine *E = nullptr;
    if (get_engine(&E) != CUTC_OK)
        return;
    std::lock_guard<std::mutex> lk(E->mu);
    int s = int2e_from_full_x(E, cudaStreamLegacy, n_grid1, n_ao, wr1, aos_data1, int2_grad1_u12,
                              int_2e_ao);
    if (s == CUTC_OK) {
        trans_inplace(int_2e_ao, n_ao * n_ao);  // A + A^T (src/build_int_2e_ao.cu:134-141)
        const cudaError_t e = cudaStreamSynchronize(cudaStreamLegacy);
        if (e != cudaSuccess) {
            cutc_set_error(CUTC_ERR_CUDA, "get_int_2e_ao: %s", cudaGetErrorString(e));
            s = CUTC_ERR_CUDA;
        }
    } else {
        cudaStreamSynchronize(cudaStreamLegacy);
    }
    report(s, "get_int_2e_ao");
}
